/*
 * omd_oracle -- CPU FP64 restatement of the Object-MD force-evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library, and only
 * as the checker.  The product (libomdg) never links or calls it.
 *
 * Each function names the reference lines it restates.  Its agreement with
 * the reference itself is pinned by tests/golden/ fixtures produced by the
 * reference's own code (oracle/ref/ref_driver, built from the reference
 * sources) -- except Tersoff, whose reference header does not compile: its
 * parity is unpinned and follows Tersoff, PRB 37, 6991 (1988), the source the
 * reference parameter file cites.
 *
 * Conventions (shared with the product):
 *   positions x[3*i+d], FP64, Angstrom; box lo/hi, periodic flags per axis;
 *   neighbour tuples (i, j, s) mean "atom j displaced by s*L is within Rv of i",
 *   with the image vector packed as code = (sx+1) + 3(sy+1) + 9(sz+1);
 *   forces eV/A, per-atom energies eV, per-atom virial r.f summed over pairs.
 */
#ifndef OMD_ORACLE_H
#define OMD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n;                  /* NumberOfData */
    double dr, off;         /* Spacing, Offset */
    int rmult;              /* Format RMULT */
    int allow_lo, allow_hi; /* OutOfRangeLower / OutOfRangeUpper given */
    double out_lo, out_hi;
    double *a, *b, *c, *d;  /* spline coefficients, d = tabulated values */
} oc_table;

/* treader.cpp:37-64: coefficients from t->d (tridiagonal solve, end rows b=5). */
void oc_table_coef(oc_table* t);
/* treader.cpp:193-229: value and derivative; returns -1 when the reference would die. */
int oc_table_read(const oc_table* t, double r, double* val, double* dval);
double oc_table_max_range(const oc_table* t);

typedef struct {
    double lo[3], hi[3];
    int periodic[3];
} oc_box;

/*
 * Canonical full neighbour set within rv (VerletList.cpp:126-199 with the
 * periodic ghost images of comhandler.cpp:288-377): for each i every (j, s)
 * with |x_i - (x_j + s L)|^2 <= rv^2, evaluated as dx = x_i - (x_j + s L)
 * and r2 = (dx*dx + dy*dy) + dz*dz in FP64, excluding (i, i, 0).  Rows are
 * sorted by (j, code).  Returns the tuple count or -1 if cap is exceeded.
 * offsets has n+1 entries (CSR).
 */
long oc_neighbors(const oc_box* box, int n, const double* x, double rv, int* offsets, int* nbr_j, int* nbr_code,
                  long cap);

/* Result arrays: f[3n], e[n], vir[n]; all overwritten. */

/* team.cpp:81-92 (density), :116-145 (embedding), :224-237 (pair force). */
int oc_eam(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j, const int* nbr_code,
           const oc_table* phi, const oc_table* edens, const oc_table* embed, double* f, double* e, double* vir,
           double* rho);

/* tpair.h:62-71: tabulated pair, r < rc strict. */
int oc_pair_table(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j,
                  const int* nbr_code, const oc_table* phi, double* f, double* e, double* vir);

/* sw.cpp:35-273 with every triplet (j<k in list order) visited once. */
typedef struct {
    double eps, A, B, p, q, sigma, a, lambda, gamma, icos0;
    int usezbl;
    double sx0, sx1, sa0, sa1, sa2, sa3;
    double z1, z2; /* atomic numbers for the ZBL core */
} oc_sw_param;
int oc_sw(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j, const int* nbr_code,
          const oc_sw_param* p, double* f, double* e, double* vir);

/* Tersoff (1988) bond order, parameter names of tables/tersoff.silicon. */
typedef struct {
    double A, B, lambda1, lambda2, lambda3, beta, n, c, d, h, R, D;
} oc_tersoff_param;
int oc_tersoff(const oc_box* box, int n, const double* x, const int* offsets, const int* nbr_j,
               const int* nbr_code, const oc_tersoff_param* p, double* f, double* e, double* vir);

/* Mixed species: per-pair-type dispatch is done by the caller; this applies
   a tabulated pair only to pairs whose types are (ta,tb) in either order. */
int oc_pair_table_typed(const oc_box* box, int n, const double* x, const int* type, int ta, int tb,
                        const int* offsets, const int* nbr_j, const int* nbr_code, const oc_table* phi, double* f,
                        double* e, double* vir);

/* Universal ZBL screened Coulomb between types (ta,tb) in either order, as
   StillingerWeber::ZBL (sw.cpp:118-146, constants sw.cpp:84-91), for r < rc,
   times the switch S(r) = 1 - t^3 (10 - 15 t + 6 t^2), t = (r - rc + width) /
   width, on [rc - width, rc] (the cut of omdg_add_zbl; the reference's ZBL
   core has none).  Adds to f, e, vir. */
int oc_zbl(const oc_box* box, int n, const double* x, const int* type, int ta, int tb, double z1, double z2,
           double rc, double width, const int* offsets, const int* nbr_j, const int* nbr_code, double* f, double* e,
           double* vir);

/* integrator.cpp:225-259 first half: v += dt/2 f/m ; x += dt v (active atoms). */
void oc_vv_kick_drift(int n, double* x, double* v, const double* f, const double* mass, double dt);
/* integrator.cpp:249-257 second half: v += dt/2 f/m. */
void oc_vv_kick(int n, double* v, const double* f, const double* mass, double dt);
/* system.cpp:1075-1094: 0.5 sum m v^2. */
double oc_kinetic(int n, const double* v, const double* mass);
/* systemgrid.cpp:129-151 + comhandler UnpackPosition: wrap owners into the box. */
void oc_wrap(const oc_box* box, int n, double* x);
/* TempController.h:78-91 Berendsen factor. */
double oc_berendsen_factor(double dt, double tau, double tset, double tnow);

#ifdef __cplusplus
}
#endif
#endif
