/*
 * omdg.h -- C ABI of libomdg, the GB300 (sm_103a) force-evaluation engine for
 * Object-MD.  Plain C types only; every call returns an int status
 * (OMDG_OK = 0, negative OMDG_E* on failure; omdg_last_error() gives text).
 *
 * One context owns one simulation box on one GPU: atoms, tables, neighbour
 * list and integrator state live in device memory; the caller owns every host
 * buffer it passes.  A context is used by one host thread at a time and all
 * its work is ordered on the context's CUDA stream.
 *
 * Atom order: the library keeps atoms sorted by linked cell internally; every
 * array passed in or out is in the caller's order (the order of
 * omdg_set_atoms), which for an Object-MD application is the enumeration
 * order nid (system.cpp:389-397).
 *
 * Each entry point names the reference interface it replaces.  Paths are
 * relative to the Object-MD source tree.
 */
#ifndef OMDG_H
#define OMDG_H

#ifdef __cplusplus
extern "C" {
#endif

#define OMDG_OK 0
#define OMDG_EINVAL (-1)        /* bad argument */
#define OMDG_ECUDA (-2)         /* CUDA runtime error */
#define OMDG_ERANGE (-3)        /* table read outside its range: TableReader::read dies (treader.cpp:199-218) */
#define OMDG_EOVERLAP (-4)      /* r^2 < 1e-6: CalcSqrDistance dies (gadget.cpp:149-159) */
#define OMDG_ENOMEM (-5)        /* device allocation failed */
#define OMDG_ESTATE (-6)        /* call out of order (e.g. no atoms yet) */
#define OMDG_EFILE (-7)         /* table / parameter file missing or malformed */
#define OMDG_ENONFINITE (-8)    /* NaN or Inf in positions or forces */

typedef struct omdg_ctx omdg_ctx;

/* ---------------------------------------------------------------- context */

/* Replaces MDSystem construction (system.h:257) for the force path. */
int omdg_create(omdg_ctx** ctx, int device);
int omdg_destroy(omdg_ctx* ctx);
const char* omdg_last_error(omdg_ctx* ctx);
/* The context's cudaStream_t, for callers that record events on it. */
int omdg_get_stream(omdg_ctx* ctx, void** stream);

/* ------------------------------------------------------------- atoms, box */

/* MDSystem::SetBox (system.cpp:849-858) + boundary.periodic (system.cpp:228-237). */
int omdg_set_box(omdg_ctx* ctx, const double lo[3], const double hi[3], const int periodic[3]);

/*
 * Atoms as the reference's Import/AtomContainer holds them (base.h:114-125):
 * x, v are n*3 FP64 (A, A/ps); type is the container id tid (0..ntypes-1);
 * mass_by_type in simulation units (amu / 9648.53397731809, container.cpp:94);
 * z_by_type the atomic numbers (used by ZBL cores).  v may be NULL (zero).
 */
int omdg_set_atoms(omdg_ctx* ctx, int n, const double* x, const double* v, const int* type, int ntypes,
                   const double* mass_by_type, const double* z_by_type);
int omdg_num_atoms(omdg_ctx* ctx, int* n);

/* Copies device state to host arrays in caller order; any pointer may be NULL.
   x, v, f are n*3; pot, vir are n (per-atom potential and virial as Atom::potential/virial). */
int omdg_get_state(omdg_ctx* ctx, double* x, double* v, double* f, double* pot, double* vir);
/* Overwrites positions / velocities (n*3 FP64, caller order).  New positions
   keep the neighbour list unless an atom moved more than skin/2 since it was
   built; the next step or force evaluation then rebuilds it.  Each call
   returns once the caller's arrays have been read.  omdg_set_state uploads
   both in one call (either may be NULL).  Pinned host arrays (cudaHostAlloc,
   cudaHostRegister) are read and written by the device directly, here and in
   omdg_get_state; other memory goes through a device staging copy. */
int omdg_set_positions(omdg_ctx* ctx, const double* x);
int omdg_set_velocities(omdg_ctx* ctx, const double* v);
int omdg_set_state(omdg_ctx* ctx, const double* x, const double* v);

/*
 * Replica mode (no single counterpart in the reference: each of its impact
 * runs is one MDSystemGrid, test/si-impact/main.cpp).  nrep independent
 * boxes in one context: replica r owns natoms[r] consecutive atoms (the
 * order omdg_set_atoms then receives), its box lo/hi (nrep x 3 each) and the
 * common periodic flags.  Every step kernel covers all replicas in one
 * launch; neighbours are only found within a replica.  Replaces omdg_set_box;
 * Tersoff and ZBL kernels.
 */
int omdg_set_replicas(omdg_ctx* ctx, int nrep, const int* natoms, const double* lo, const double* hi,
                      const int periodic[3]);
/* Kinetic and potential energy of every replica (MeasureKinetic/MeasurePotential per box). */
int omdg_replica_ledger(omdg_ctx* ctx, int nrep, double* kinetic, double* potential);

/* --------------------------------------------------------- force kernels */

/*
 * TForceEAM(table) + its auto-created TEmbedding (team.cpp:166-237, :37-145):
 * reads the PAIR, EDENS and EMBED sections of the Object-MD table file with
 * TableReader semantics (treader.cpp:37-264).  type_a == type_b only.
 */
int omdg_add_eam(omdg_ctx* ctx, int type_a, int type_b, const char* table_file);

/* TForcePair(table) (tpair.h:38-71); fp64 != 0 evaluates it in FP64 end to end. */
int omdg_add_pair_table(omdg_ctx* ctx, int type_a, int type_b, const char* table_file, int fp64);

/* StillingerWeber(material) (sw.cpp:35-273), parameters from an sw.* file.
   Every triplet is evaluated (the reference's sw.cpp:261 guard is not reproduced). */
int omdg_add_sw(omdg_ctx* ctx, int type_a, int type_b, const char* param_file);

/* Tersoff(material) (include/potential/tersoff.h:104), tersoff.* keys;
   the bond-order form of Tersoff, PRB 37, 6991 (1988). */
int omdg_add_tersoff(omdg_ctx* ctx, int type_a, int type_b, const char* param_file);

/* Universal ZBL screened Coulomb pair (sw.cpp:118-146 form) between two types,
   cut at rc with a smoothing switch over [rc - width, rc]. */
int omdg_add_zbl(omdg_ctx* ctx, int type_a, int type_b, double rc, double width);

/* Max cut radius over all kernels (integrator.cpp:108-113). */
int omdg_max_cut_radius(omdg_ctx* ctx, double* rc);

/* --------------------------------------------------------- neighbour list */

/*
 * VerletList / VerletListFull with comm.tolerance `skin` (absolute) as the
 * MDSystemGrid radius tolerance (systemgrid.cpp:610-617): Rv = rc_max + skin.
 * rebuild_every > 0 rebuilds every that many steps (comm.refresh);
 * rebuild_every == 0 rebuilds when any atom moved more than skin/2 since the
 * last build (displacement trigger).
 */
int omdg_set_neighbor(omdg_ctx* ctx, double skin, int rebuild_every);
int omdg_build_neighbors(omdg_ctx* ctx);
/*
 * Canonical neighbour tuples of the current list, caller order: for atom i
 * the entries (j, code) with code = (sx+1) + 3(sy+1) + 9(sz+1) the image of
 * j.  offsets has n+1 entries; j/code have capacity `cap`; *count receives
 * the number of tuples (also when cap is too small, then OMDG_EINVAL).
 */
int omdg_get_neighbors(omdg_ctx* ctx, int* offsets, int* nbr_j, int* nbr_code, long cap, long* count);

/* ----------------------------------------------------- force / integration */

/* MDIntegrator::Iterate (integrator.cpp:203-216): one force evaluation. */
int omdg_compute_forces(omdg_ctx* ctx);

/* MDIntegrator(dt) / time.step (integrator.cpp:116-122). */
int omdg_set_timestep(omdg_ctx* ctx, double dt);

/*
 * nsteps of RunKernel (system.cpp:964-983): Integrate (integrator.cpp:225-259),
 * MeasurePotential/MeasureKinetic, POST_INTEGRATION modifies.  The first call
 * runs FirstRun (system.cpp:860-873) first; with reference_first_step != 0 it
 * zeroes the forces afterwards as the reference does.
 */
int omdg_step(omdg_ctx* ctx, int nsteps);
/* omdg_step without the final wait: enqueues nsteps on the context stream.
   omdg_sync waits for them, checks the device status and updates the ledger.
   When a list rebuild inside the queued steps needs longer rows than were
   allocated (the reference grows its rows instead, VerletListFull.cpp:127-136),
   the steps after it are discarded: omdg_sync restores the state that rebuild
   started from, grows the rows, redoes that step and replays the rest, so the
   result equals a run with ample rows bit for bit (not with the two-temperature
   model, whose electron state is outside the restored copy: there the overflow
   is reported as OMDG_ESTATE). */
int omdg_step_async(omdg_ctx* ctx, int nsteps);
int omdg_sync(omdg_ctx* ctx);
/* One MD call driven from host arrays (caller order, n*3 FP64; any pointer
   may be NULL): uploads x_in / v_in as omdg_set_state does, runs nsteps as
   omdg_step does, and writes the last step's positions, velocities and
   forces as omdg_get_state does; returns once they are in place.  With
   pinned output arrays and no thermostat, the last step writes x and f to
   the host while its force and kick kernels run. */
int omdg_step_io(omdg_ctx* ctx, const double* x_in, const double* v_in, int nsteps, double* x_out, double* v_out,
                 double* f_out);
int omdg_set_first_step_mode(omdg_ctx* ctx, int reference_first_step);

/*
 * Energy ledger of the last completed step: kinetic, potential (non-ghost,
 * active atoms), base potential of FirstRun and virial/2
 * (system.cpp:1060-1094, :971).  Energy = kinetic + potential - base.
 */
int omdg_ledger(omdg_ctx* ctx, double* kinetic, double* potential, double* base_potential, double* virial);
/* Per-step ledger rows (kinetic, potential) of the last omdg_step call, up to cap rows. */
int omdg_ledger_history(omdg_ctx* ctx, double* kinetic, double* potential, int cap, int* rows);

/* TempController(T, tau) (TempController.h:51-91); tau <= 0 removes it.
   The temperature is 2/3 KE / (N k_B) over the box's atoms. */
int omdg_set_thermostat(omdg_ctx* ctx, double temperature, double tau);

/*
 * Reference-compatibility switches for behaviour of the reference that this
 * library does not take by default:
 *   "first_step_zero_force"    FirstRun zeroes the forces it computed, so the
 *                              first half kick uses f = 0 (system.cpp:872);
 *                              same as omdg_set_first_step_mode; default on.
 *   "thermostat_counts_ghosts" TempController divides the kinetic energy by
 *                              GetTotalAtom(), which on the periodic
 *                              MDSystemGrid counts the ghost images too
 *                              (system.h:337); default off.
 */
int omdg_set_compat(omdg_ctx* ctx, const char* key, int on);

/* Number of neighbour-list builds so far and of kernel launches issued by the last omdg_step. */
int omdg_stats(omdg_ctx* ctx, long* rebuilds, long* launches);
/* Replica mode: the list builds of each replica so far.  Inside steps a replica is re-sorted and its rows rebuilt
   only when one of its own atoms moved more than skin/2 since its last build, as when it runs alone; a periodic
   rebuild (rebuild_every), a state upload or an eager build takes all of them. */
int omdg_replica_builds(omdg_ctx* ctx, int* builds, int nrep);
/*
 * No reference counterpart (the reference has one scalar loop per potential).
 * Centres the last Stillinger-Weber or Tersoff force pass queued for the
 * dense second pass (k_sw_wide / k_tersoff_wide: more in-cutoff neighbours
 * than the register path holds, 8 for SW and 4 for Tersoff).  Synchronous.
 */
int omdg_wide_centres(omdg_ctx* ctx, int* count);

/*
 * No reference counterpart (the reference's EAM loops over its half list,
 * team.cpp:224-237).  The tiles of the last list build for the tiled EAM
 * passes (blocks of cells whose halo is staged in shared memory), and how
 * many of them fit the staging capacity (launch key tile_cap; the others
 * take the gather path).  Both 0 when the last build wrote no tile slots.
 * Synchronous.
 */
int omdg_tile_counts(omdg_ctx* ctx, int* tiles, int* staged);

/*
 * Launch shapes (no reference counterpart: the reference is scalar C++).
 * Keys: "eam_block", "eam_lanes" (threads per atom), "eam_stage" (spline
 * knots in shared memory), "eam_ctas_per_sm", "pair_block", "pair_lanes",
 * "tb_lanes" (the three-body candidate's lanes, which set the neighbour slice
 * height; its kernels run one thread per centre), "tb_block" (kept for
 * callers that set it; the three-body kernels run 128-thread blocks),
 * "nbr_hshift" (log2 of the neighbour slice height),
 * "build_lanes" (list build: 0 cell CTAs, else threads per atom), "io_blocks"
 * (blocks of omdg_step_io's downloads beside the step's kernels), "nbr_capacity"
 * (row capacity of the next first list build; 0 sizes it from the density;
 * rows grow by themselves when a build needs more), "tb_persistent" (the
 * Tersoff register pass as one resident grid), "fuse_kick" (the step's second
 * half-kick in the EAM force kernel's epilogue), "eam_tile" (the tiled EAM
 * passes: one CTA per block of "tile_x" x "tile_y" x "tile_z" cells, at most
 * "tile_cap" staged atoms; changing any of them rebuilds the list), "nn_fused"
 * (the surrogate's descriptors computed inside its network kernel).  All are
 * 0/1 switches or sizes; results agree across them within FP32 summation order.
 */
int omdg_set_launch(omdg_ctx* ctx, const char* key, int value);
int omdg_get_launch(omdg_ctx* ctx, const char* key, int* value);
/*
 * Times the force kernels of the current system under candidate launch
 * shapes (CUDA events, best of `reps` force evaluations each) and keeps the
 * fastest.  best_ms receives its time per force evaluation.
 */
int omdg_autotune(omdg_ctx* ctx, int reps, double* best_ms);

/* Per-kernel CUDA-event timing of subsequent omdg_step calls (tracing). */
int omdg_set_profiling(omdg_ctx* ctx, int on);
/* name_buf receives "name;name;..."; ms[] the summed milliseconds, calls[] the launch counts. */
int omdg_kernel_times(omdg_ctx* ctx, char* name_buf, int name_cap, double* ms, long* calls, int cap, int* nkern);

/* ------------------------------------- local thermodynamics, two-temperature */

/*
 * ThermoDetector in intensive mode (include/detect/ThermoDetector.h:176-237):
 * after every step, each atom's local centre-of-mass velocity, temperature
 * and density over itself and its neighbours within ercut (<= 0: the largest
 * cutoff of the force kernels, as the reference's default).
 */
int omdg_set_thermo_detector(omdg_ctx* ctx, int on, double ercut);
/* Local temperature (K), density (1/A^3) and centre-of-mass velocity (n*3) per atom, caller order; may be NULL. */
int omdg_local_thermo(omdg_ctx* ctx, double* temperature, double* density, double* vcm);
/*
 * TTM_Homogen (include/misc/TTM_Homogen_SCNA.h): a homogeneous electron
 * temperature coupled to the lattice by scaling-corrected velocity rescaling
 * about each atom's local centre of mass.  table_file holds the
 * ELECTRON_PHONON_COUPLING and ELECTRON_HEAT_CAPACITY sections (each with a
 * Constant); atom_volume in A^3; electron_temperature < 0 starts from the
 * lattice temperature; coupling starts once the elapsed time exceeds
 * pulse_offset (ps).  Turns the detector on.
 */
int omdg_set_ttm(omdg_ctx* ctx, const char* table_file, double atom_volume, double electron_temperature,
                 double pulse_offset);
/* Electron temperature, integrated electron energy, integrated energy per atom given to the lattice, and the mean
   local lattice temperature (the "e_temp:", "int_Een:", "int_Aen:" slots and GetTemperatureAvg). */
int omdg_ttm_state(omdg_ctx* ctx, double* electron_temperature, double* int_een, double* int_aen,
                   double* lattice_temperature);

/* ------------------------------------------------------ neural surrogate */

/*
 * No counterpart in the reference.  An atom-centred network stands in for
 * Tersoff Si: 32 descriptors per atom (16 radial, 16 angular; cutoff from
 * the model, 3.2 A by default), a 32-64-64-1 tanh network evaluated on the
 * tensor cores (BF16 weights and activations, FP32 accumulation) and forces
 * from the analytic gradient.  model_file is written by omdg_nn_save.  With
 * tersoff_fallback (a Tersoff parameter file, as for omdg_add_tersoff) every
 * atom whose descriptors leave the training range takes its energy and
 * forces from Tersoff instead; NULL disables the fallback.  A model whose
 * angular terms keep the default layout (zeta 1, 1, 2, 2, 4, 4, 8, 8 twice,
 * lambda alternating +1, -1) runs descriptor and force kernels specialised
 * for it; any other layout runs general kernels (the same terms, without
 * the powers shared across terms).
 */
int omdg_add_nn(omdg_ctx* ctx, int type_a, int type_b, const char* model_file, const char* tersoff_fallback);
/* Atoms handed to the Tersoff fallback in the last force evaluation. */
int omdg_nn_fallback_atoms(omdg_ctx* ctx, long* atoms);

/*
 * Training on one GPU (no reference counterpart).  A dataset is nconf
 * periodic configurations: natoms[c] atoms each, positions x (sum natoms x 3,
 * FP64), box lengths box_len (nconf x 3, each at least twice the cutoff),
 * reference total energies (nconf) and forces (sum natoms x 3).  Parameters
 * are one FP32 vector of 6337 values: W1[64x32] b1[64] W2[64x64] b2[64]
 * w3[64] b3.  Loss: wE mean_c ((E_c - E_ref)/N_c)^2 + wF mean (F - F_ref)^2.
 */
typedef struct omdg_nn omdg_nn;
int omdg_nn_create(omdg_nn** nn, int device);
int omdg_nn_destroy(omdg_nn* nn);
const char* omdg_nn_last_error(omdg_nn* nn);
/* Descriptor parameters (16 radial: rs, eta_r; 16 angular: zeta, lambda, eta_a), before the dataset; the defaults are
   rs on [1.6, 3.2] A with eta_r = 1/(2 h^2), and (eta_a in {0, 0.3}) x (zeta in {1, 2, 4, 8}) x (lambda in {1, -1}). */
int omdg_nn_set_descriptors(omdg_nn* nn, const float* rs, const float* eta_r, const int* zeta, const float* lambda,
                            const float* eta_a);
/* Descriptor cutoff rc and the inner radius rin where its switch starts (before the dataset): f_c = 1 up to rin and
   (cos(pi (r - rin) / (rc - rin)) + 1) / 2 on (rin, rc).  The default is rc = 3.2 A, rin = 0; rin = R - D and
   rc = R + D give Tersoff's own switch (tersoff.h:183).  OMDG_EINVAL unless 0 <= rin < rc. */
int omdg_nn_set_cutoff(omdg_nn* nn, float rc, float rin);
int omdg_nn_set_dataset(omdg_nn* nn, int nconf, const int* natoms, const double* x, const double* box_len,
                        const double* energy, const double* forces);
/* relative != 0 weights each configuration's force residual by (mean square force of the dataset) / (its own), so
   that every configuration counts by its relative error; 0 (the default) is the plain mean square. */
int omdg_nn_set_force_weighting(omdg_nn* nn, int relative);
/* Per-atom reference energies (sum natoms, e.g. a force kernel's per-atom potential): the energy term becomes
   wE mean_i (E_i - E_i^ref)^2 over the batch atoms.  NULL restores the per-configuration total-energy term. */
int omdg_nn_set_atom_energies(omdg_nn* nn, const double* e_atom);
/* Raw descriptors of the dataset (sum natoms x 32). */
int omdg_nn_descriptors(omdg_nn* nn, float* G, long count);
/* Mean, deviation and range of the dataset's descriptors become the input scaling and the fallback range. */
int omdg_nn_normalize_from_dataset(omdg_nn* nn);
int omdg_nn_set_normalization(omdg_nn* nn, const float* mu, const float* sigma, const float* gmin, const float* gmax);
int omdg_nn_get_normalization(omdg_nn* nn, float* mu, float* sigma, float* gmin, float* gmax);
int omdg_nn_set_weights(omdg_nn* nn, const float* params, long count);
int omdg_nn_get_weights(omdg_nn* nn, float* params, long count);
/* Loss and dL/dparams (FP32 kernels) over configurations [conf0, conf0 + nconf). */
int omdg_nn_gradient(omdg_nn* nn, int conf0, int nconf, double wE, double wF, double* loss, float* grad);
/*
 * Adam (beta 0.9/0.999) over shuffled batches of batch_confs configurations,
 * learning rate lr in the first epoch decaying by a cosine to lr_final in the
 * last (lr_final = lr: constant); epoch_loss (may be NULL) receives the mean
 * batch loss of each epoch.
 */
int omdg_nn_train(omdg_nn* nn, int epochs, int batch_confs, double lr, double lr_final, double wE, double wF,
                  unsigned seed, double* epoch_loss);
/* Per-atom energies and forces of configurations [conf0, conf0 + nconf) with the tensor-core network
   (BF16 operands), or with fp32 != 0 the FP32 kernels training uses. */
int omdg_nn_predict(omdg_nn* nn, int conf0, int nconf, int fp32, double* energy_per_atom, double* forces);
int omdg_nn_save(omdg_nn* nn, const char* path);
int omdg_nn_load(omdg_nn* nn, const char* path);

/* ------------------------------------------------------- bounded waits */

/*
 * No reference counterpart (the reference has no device code).  Every wait
 * of the tensor-core kernels (an mbarrier for a bulk copy or an MMA) polls at
 * most `polls` times (0 restores the default, 4,194,304); when it gives up,
 * the CTA waits for its own copy or MMA to finish, records ERR_TIMEOUT, which
 * the calling entry point returns as OMDG_ECUDA "a bounded device wait
 * expired", and returns.  Process-wide; takes effect at the next launch.
 */
int omdg_set_wait_polls(int polls);

/*
 * No reference counterpart.  Makes one kind of bounded wait run out on the
 * current device and returns its status word in *status (ERR_TIMEOUT = 32
 * when it gave up): which 0 = an mbarrier that nothing arrives at, in a CTA
 * holding TMEM as the tensor-core kernels do; which 1 = a grid barrier whose
 * arrival count the grid can never reach.  Neither hangs nor faults: the
 * kernel returns after `polls` polls and the device stays usable.
 */
int omdg_selftest_wait(int which, int polls, unsigned* status);

/* ------------------------------------------------- allocation-free counting */

/*
 * No counterpart in the reference.  Per-atom neighbour counts for positions
 * that already live in the caller's device memory, for callers that cannot
 * let a library allocate device memory: a host code whose own pool allocator
 * has reserved the GPU's memory (a cudaMalloc would fail or fragment it), or
 * one that keeps other streams busy (cudaFree synchronises the device).  This
 * call allocates nothing: no cudaMalloc/cudaFree, no allocating library call.
 *
 * x: device pointer, n*3 FP64 positions (any order; periodic axes are wrapped
 * into the box on the fly); count: device pointer, n ints.  The result equals
 * the per-atom neighbour count of the Verlet list (owners and periodic images
 * with r^2 <= rcut^2, computed as omdg_build_neighbors does with Rv = rcut).
 * Work is queued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) of the current device and the call returns without waiting.
 *
 * Limits: n <= OMDG_STATIC_MAX_ATOMS; every periodic axis longer than 3 rcut
 * (cells are at least rcut (1 + 1e-12) wide, so an axis of exactly 3 rcut is
 * rejected); the cell grid is coarsened to OMDG_STATIC_MAX_CELLS cells when the box
 * holds more.  Scratch is one fixed __device__ array of about 1.4 MB per
 * device, shared by every call: calls that overlap in time (on different
 * streams, or from several host threads at once) race on it and give wrong
 * counts; calls queued on one stream do not.  The cell counters that must
 * start at zero are cleared by each call itself.  The first call on a device
 * looks the scratch address up (cudaGetSymbolAddress, which also loads the
 * module's kernels), so make it once at setup, with that device current and
 * before any stream capture.  That address is kept for the life of the
 * process and never looked up again: after cudaDeviceReset (or anything else
 * that destroys the device's primary context) it is stale, so do not call
 * this entry point on that device again in the same process.
 *
 * Returns OMDG_OK, OMDG_EINVAL (bad argument, box too small), OMDG_ERANGE
 * (n above the limit) or OMDG_ECUDA; err (may be NULL) receives the message.
 */
#define OMDG_STATIC_MAX_ATOMS 131072
#define OMDG_STATIC_MAX_CELLS 32768
int omdg_count_neighbors_static(const double* x, int n, const double lo[3], const double hi[3], const int periodic[3],
                                double rcut, int* count, void* stream, char* err, int err_len);

/* ------------------------------------------------- impact-run modifies */

/*
 * The modifies of the reference's impact runs (test/si-impact/main.cpp:73-76)
 * on the device.  Modifies act on atom groups (AtomGroup selections such as
 * SelectType + SelectInverseBox, main.cpp:55-65): bit g of member[i] puts
 * caller atom i in group g (0..7); group -1 in the calls below means every
 * atom.  Membership is fixed, as the reference selects at setup.
 */
int omdg_set_groups(omdg_ctx* ctx, const unsigned char* member);
/* FLAG_ACTIVE per atom (Atom::flag bit 0, base.h:230; SetActive, base.h:285):
   inactive atoms are not integrated (integrator.cpp:233, :250), not listed
   (VerletList.cpp:97) and not measured (system.cpp:1067, :1085). */
int omdg_set_active(omdg_ctx* ctx, const int* active);
int omdg_get_active(omdg_ctx* ctx, int* active);
/* ForceDamper (ForceDamper.h:30-36): after the forces, f -= factor * v. */
int omdg_add_force_damper(omdg_ctx* ctx, int group, double factor);
/* CoordClamp (CoordClamp.h:23-42): after the forces, f = v = 0 on the axes
   CoordClamp::Init selects from `axes`; it tests `if(saxis.find('x'))`, so an
   axis is clamped when its letter is absent or not first ("xyz": y and z). */
int omdg_add_coord_clamp(omdg_ctx* ctx, int group, const char* axes);
/* RangeLimiter (RangeLimiter.h:21-54): after each step, group atoms beyond
   the box -/+ border are deactivated. */
int omdg_add_range_limiter(omdg_ctx* ctx, int group, double border);
/* DynamicTimeStep(maxpath, max, update) (DynamicTimeStep.h:44-70): every
   `update` steps TimeStep = min(maxpath / (1.1 sqrt(SqrMaxVelocity)), max),
   SqrMaxVelocity over active atoms (system.cpp:1075-1094); evaluated on the
   device between steps.  TimeStep starts at max (Init with no velocity). */
int omdg_set_dynamic_timestep(omdg_ctx* ctx, double maxpath, double max_dt, int update);
/* EnergySource, pulse mode (EnergySource.h:78-131): from ElapsedTime >= start
   (its first call there only arms it) until start + width, each step scales
   every active atom's velocity by sqrt(1 + 2 delta / (m v^2)), delta =
   energy * dt / width (width at least dt), skipping v^2 < (1e-6 |v|max)^2.
   start must be > 0 (start = 0 draws random velocities, SetKineticEnergy);
   not with DynamicTimeStep (the reference refuses it) nor with the Berendsen
   thermostat (its factor waits in the step state until the next kick). */
int omdg_add_energy_source(omdg_ctx* ctx, double energy, double start, double width);
/* Integrator->TimeStep and ElapsedTime (system.cpp:979) as the device has them. */
int omdg_get_timestep(omdg_ctx* ctx, double* dt, double* elapsed);

/* ------------------------------------------------------------------ output */

/* DumpAtoms write modes (container.h:34-45). */
#define OMDG_WM_APPEND 1
#define OMDG_WM_VELOCITY 2
#define OMDG_WM_FORCE 4
#define OMDG_WM_DEADATOM 8
#define OMDG_WM_BARE 16
#define OMDG_WM_GHOST 32
#define OMDG_WM_POTENTIAL 64
#define OMDG_WM_VIRIAL 128
#define OMDG_WM_TID 256
#define OMDG_WM_GID 512
#define OMDG_WM_NID 1024
#define OMDG_WM_ZIP 2048

/* AtomContainer::DumpAtoms (container.cpp:417-519), the Object-MD data file
   of the context's atoms from device state, in caller (nid) order: unless
   WM_BARE or WM_APPEND the header (Box, the caller's info lines as "#<line>",
   Material, Fields), then per active atom (all with WM_DEADATOM) x y z fixed
   with posprec digits and the mode's fields in scientific with valprec
   (id = type, gid from the caller or 0, nid = caller index).  WM_ZIP (gzip)
   is refused; there are no ghost atoms to include. */
int omdg_dump_atoms(omdg_ctx* ctx, const char* path, int mode, int posprec, int valprec, const char* material,
                    int ninfo, const char* const* info, const int* gid);
/* ThermoDetector's data file (ThermoDetector.h:100-115, 232-420, through
   DataDumper::Measure, DataDumper.h): the detector (omdg_set_thermo_detector)
   must have run on the current state (a step or omdg_compute_forces).  Info
   lines: "$ DetectorVolume" (4/3 pi ercut^3), the caller's lines, then
   "$ Temperature <T> K (kinetic)", "$ Pressure <P> GPa" (the system's, about
   the centre-of-mass velocity, over the active atoms' bounding box) and
   "$ Time <elapsed>"; per atom the columns temp press dens after x y z, in
   aux_format (NULL: "%0.5e"), then the mode's fields as omdg_dump_atoms.
   summary (may be NULL) receives 5 values: system temperature (K), system
   pressure (GPa), and the averages of the local temperature, density and
   pressure (ThermoDetector's GetTemperatureAvg, GetDensityAvg,
   GetPressureAvg). */
int omdg_dump_thermo(omdg_ctx* ctx, const char* path, int mode, int posprec, int valprec, const char* material,
                     int ninfo, const char* const* info, const char* aux_format, double* summary);
/* SysMonitor (SysMonitor.h): appends the md.out lines of the steps completed
   by the last omdg_step / omdg_sync with Step % every == 0 and Step != 0:
   "Step ElapsedTime TimeStep Ek Ep E" with SysMonitor's formats, from the
   device ledger; with the thermo detector on, also ThermoDetector's slots
   temp: avtemp: pres: avpres: (system temperature, average local
   temperature, system pressure, average local pressure; %0.3E), measured
   on the device after every step.  header != 0 truncates the file and
   writes the label line. */
int omdg_monitor_append(omdg_ctx* ctx, const char* path, int every, int header);

/* ------------------------------------------------------------ checkpoints */

/*
 * Binary checkpoint in the reference's own format, so that a run resumes
 * here or hands off to the CPU code and back (MDSystem::SaveSimulation /
 * LoadSimulation, system.cpp:726-827; AtomContainer::Save / Load,
 * container.cpp:554-680).  File order:
 *   "OMD (c) Y ROSANDI" and a time stamp, 32 bytes each (NUL padded);
 *   the SaveVariables block (system.cpp:656-668, omdg_sim_vars below);
 *   int count of restart variables, each a label and a value string;
 *   int count of containers and their names, 32 bytes each;
 *   "== END OF CONFIG HEADER ===" (32 bytes);
 *   per container: "$ATOMCONTAINER:" (32 bytes), the name, material, file
 *   and parameter strings, id, M, Z, Value, posprec, valprec, write_mode,
 *   the atom count and the raw Atom records (base.h:114-125).
 * A string is an int length (with the NUL) and its bytes.  Host byte order
 * and the LP64 layout, on which x86-64 and aarch64 agree.
 */
#define OMDG_AUXVAR 16 /* MAXAUXVAR (config.h:26) */
#define OMDG_FLAG_ACTIVE 1 /* FLAG_ACTIVE (base.h:230) */

typedef struct omdg_sim_vars { /* MDSystem::SaveVariables, in file order */
    long long begin_time;      /* SimBeginTime (time_t) */
    int step;                  /* Step */
    int pboundary;             /* PBoundary: 1 x | 2 y | 4 z (system.h:44-46) */
    double energy, kinetic, virial, potential, base_potential, elapsed_time;
    double box[12]; /* SysBox: x0 x1 y0 y1 z0 z1 lx ly lz hlx hly hlz (base.h:54-60) */
    int write_mode;
} omdg_sim_vars;

typedef struct omdg_container_desc { /* a container's saved header (container.cpp:566-581) */
    char name[256], material[256], filename[256], param[1024];
    int id;                         /* the tid of its atoms */
    double mass, z, value;          /* M (simulation units), Z, Value */
    int posprec, valprec, write_mode;
    int natoms;                     /* its atoms: the next natoms records */
} omdg_container_desc;

typedef struct omdg_atom_record { /* Atom (base.h:114-125), 232 bytes */
    int tid, gid, nid, flag;
    double x, y, z, vx, vy, vz, fx, fy, fz, potential, virial;
    double aux[OMDG_AUXVAR];
} omdg_atom_record;

/* Host only (no device work): write a checkpoint from caller arrays.  stamp
   NULL takes ctime(now) as the reference does; labels/values are nvar
   restart-variable strings (DataSlot label and AsString, system.cpp:743-748);
   atoms holds the containers' records back to back. */
int omdg_checkpoint_write(const char* path, const char* stamp, const omdg_sim_vars* vars, int nvar,
                          const char* const* labels, const char* const* values, int ncont,
                          const omdg_container_desc* cont, const omdg_atom_record* atoms, char* err, int err_len);
/* Host only: the counts, to size omdg_checkpoint_read's arrays. */
int omdg_checkpoint_info(const char* path, int* ncont, int* natoms, int* nvar, char* err, int err_len);
/* Host only: read everything.  stamp gets 32 bytes; the restart variables
   come back in var_buf as label NUL value NUL pairs. */
int omdg_checkpoint_read(const char* path, omdg_sim_vars* vars, char* stamp, int ncont_cap, omdg_container_desc* cont,
                         int natom_cap, omdg_atom_record* atoms, char* var_buf, int var_buf_len, char* err,
                         int err_len);

/* MDSystem::SaveSimulation (system.cpp:767-771) from the context's state.
   Atoms go out in caller order, container after container (cont[k].natoms
   each, summing to the atom count): tid = the atom's type, nid = its caller
   index, gid and flag from the caller (NULL: 0 and OMDG_FLAG_ACTIVE), aux
   from the caller (n * OMDG_AUXVAR, NULL: zeros); x, v, f, potential and
   virial from the device; Step, the last ledger row (E = K + P - P0), P0,
   the elapsed time (sum of the steps' dt, system.cpp:979) and the box from
   the context. */
int omdg_save_simulation(omdg_ctx* ctx, const char* path, int ncont, const omdg_container_desc* cont, const int* gid,
                         const int* flag, const double* aux, int nvar, const char* const* labels,
                         const char* const* values);
/* CONTINUE_MODE (system.cpp:1004-1019, LoadSimulation): box and periodicity
   from SysBox and PBoundary, atoms in file order with type = tid (each
   type's mass and Z from the container whose id it is), velocities, and the
   stored forces for the first half-kick (no FirstRun); Step, P0 and the
   elapsed time continue from the file.  Potentials may be added before or
   after.  cont (cap entries, may be NULL) receives the container headers. */
int omdg_load_simulation(omdg_ctx* ctx, const char* path, int cap, omdg_container_desc* cont, int* ncont);

/* ------------------------------------------------------------------ finite-difference heat solver
   FDTDSolver (include/misc/fdtd.hpp, src/omd/fdtd.cpp), single rank, the cells on the device.  The grid is
   nx x ny x nz cells (nz <= 2 makes it 2D, fdtd.cpp:58-59), cell (i, j, k) at index k nx ny + i + j nx.
   symbol: the symbol map of SetSymbolMap (fdtd.cpp:450-477): "<chars> <flags>" pairs, flags one character per
   face (left right top bottom [near far]): '+' occupied, 'p' periodic, anything else empty.  map: one character
   per cell (SetMap, fdtd.cpp:479-488); a character outside the symbol map marks a cell the face loop skips.
   Conductivity and capacity start at 1, the cell vector and the source at 0 (fdtd.cpp:186-204).
   On failure *fd may still be set: read omdg_fdtd_last_error, then omdg_fdtd_destroy it. */
typedef struct omdg_fdtd omdg_fdtd;
int omdg_fdtd_create(omdg_fdtd** fd, int device, int nx, int ny, int nz, const char* symbol, const char* map);
int omdg_fdtd_destroy(omdg_fdtd* fd);
const char* omdg_fdtd_last_error(omdg_fdtd* fd);
int omdg_fdtd_set_timestep(omdg_fdtd* fd, double dt);   /* SetTimestep (fdtd.cpp:422-425) */
int omdg_fdtd_set_spacestep(omdg_fdtd* fd, double h);   /* SetSpacestep (fdtd.cpp:427-433): 1/h^2 */
/* which 0: SetCell (the cell vector, now); 1: SetSource; 2: SetConductivity; 3: SetCapacity (fdtd.hpp:123-133):
   the string is kept and re-applied before every step (sync_data, fdtd.cpp:599-603).  Tokens: "<chars> <value>"
   (every cell with one of the map characters, '*' all) or "@ i,j,k=<value>" / "@ i,j,k,i2,j2,k2=<value>" (one
   cell or a block), a value optionally followed by ":t0" or ":t0:t1" (the steps it applies in; a token is dropped
   for good once a step falls outside its range, AssignArray, fdtd.cpp:528-592).  A '{...}' value is a muParser
   expression, which is not built: OMDG_EINVAL. */
int omdg_fdtd_assign(omdg_fdtd* fd, int which, const char* str);
/* Step(n) (fdtd.cpp:671-689): per step the kept strings, one Solve (fdtd.cpp:605-668) on the device, step + 1. */
int omdg_fdtd_step(omdg_fdtd* fd, int n);
/* which 0: the cell vector, 1: the source the next step starts from, 2: conductivity, 3: capacity, 4: the
   external vector; n must be nx ny nz. */
int omdg_fdtd_get(omdg_fdtd* fd, int which, double* out, long n);
/* GetExtVector() written by the caller: E for the next solve, which clears it. */
int omdg_fdtd_set_ext(omdg_fdtd* fd, const double* e, long n);
int omdg_fdtd_info(omdg_fdtd* fd, int* nx, int* ny, int* nz, int* step);
/* The two-temperature model with the electron temperature on a grid's cells (the coupling include/misc/
   TTM_Diffusion.h:41,134 sets out to make with FDTDSolver; that header does not compile).  After omdg_set_ttm
   (tables, atom volume, pulse offset; its electron_temperature is not used: the grid's cell vector is Te, a
   negative cell taking its cell's lattice temperature at the first active step), every step first sums the
   detector temperatures of the atoms in each cell (cell (i, j, k) covers origin + h [i, i+1) x [j, j+1) x
   [k, k+1), periodic axes wrapped into the box; a 2D grid spans every z) into the lattice temperature Ta, sets
   E = -G0 G(Te) (Te - Ta) for the cells holding atoms and cap = C0 Ce(Te), runs one solve with the MD time step,
   and rescales each atom's velocity about its local centre of mass with its cell's new Te, as the scalar model
   does (TTM_Homogen_SCNA.h:272-330).  The grid's kept strings must be unranged (no ":t0:t1"): the coupled step
   replays on the device.  While coupled the grid takes no omdg_fdtd_step, assign, set_ext or destroy; read its
   cell vector after omdg_sync.  grid = NULL detaches.  omdg_ttm_state's electron temperature and integrated
   electron energy are not kept in this mode. */
int omdg_set_ttm_grid(omdg_ctx* ctx, omdg_fdtd* grid, const double* origin);

#ifdef __cplusplus
}
#endif
#endif
