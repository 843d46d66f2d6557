// The finite-difference heat solver (FDTDSolver, include/misc/fdtd.hpp and
// src/omd/fdtd.cpp) on the device: the grid object behind the omdg_fdtd_*
// entry points and the two-temperature model's electron-temperature field.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "omdg_internal.h"

namespace omdg {

// CellBoundary (fdtd.hpp:31-35): per map symbol, the exchange flag of each
// face (0 empty, 1 occupied, 2 periodic), left right top bottom near far.
struct FDBound {
    char sym;
    int l, r, t, b, n, f;
};

// Exchange directions of one cell, as Solve visits them (fdtd.cpp:615-658).
enum : uint8_t { FD_R = 1, FD_L = 2, FD_B = 4, FD_T = 8, FD_N = 16, FD_F = 32 };

// Device arrays of one grid.  A is the cell vector (two buffers: the solve
// reads the old one and writes the other), S the source pattern of the
// current step, E the external vector (zeroed by each solve), con and cap
// the conductivity and capacity, map the symbol index per cell (-1 for a
// character outside the symbol map) and mask the exchange directions.
struct FDDev {
    int nx, ny, nz, dim;
    double dt, h2inv;
    const int* map;
    const uint8_t* mask;
    const double* K;  // face conductances: x faces [0, dim), y faces [dim, 2 dim), z faces [2 dim, 3 dim)
    const double* cap;
    double* S;
    double* E;
    int keep_S;  // coupled: S is the kept strings' fixed pattern, not cleared by the solve
    // coupled to the atoms (a replayed step graph): the mask chosen on the
    // device from the solve count, and the step skipped while the model is
    // not active; null for host-driven steps
    const uint8_t* mask_first;
    const uint8_t* mask_later;
    const int* solves;
    const int* active;
};

struct FDGrid {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int nx = 0, ny = 0, nz = 0, dim = 0;
    int step = 0;                        // FDTDSolver::step
    double timestep = 1.0, spacestep = 1.0, h2inv = 1.0;
    std::vector<FDBound> bound;          // symbol map (SetSymbolMap)
    std::vector<int> map;                // SetMap
    std::vector<uint8_t> mask_first;     // exchange directions at the first solve
    std::vector<uint8_t> mask_later;     // ... and at every later one (fdtd.cpp:287-295 clears flags)
    int solves = 0;
    std::string str_src, str_con, str_cap;  // assignment strings kept for sync_data
    std::vector<double> hA, hS, hcon, hcap; // host images of the assigned arrays
    bool dirty_S = true, dirty_con = true, dirty_cap = true;  // the host image changed since the last upload
    bool s_any = false;                  // hS holds a non-zero value (cleared after each solve)
    double* dA[2] = {nullptr, nullptr};
    int cur = 0;                         // dA[cur] holds the cell vector
    double *dS = nullptr, *dE = nullptr, *dcon = nullptr, *dcap = nullptr;
    double* dK = nullptr;                // face conductances from dcon (3 x dim), refreshed with it
    int* dmap = nullptr;
    uint8_t* dmask[2] = {nullptr, nullptr};  // first, later
    bool coupled = false;                // stepped by a context's two-temperature model
};

int fd_fail(FDGrid* g, int code, const std::string& msg);
// Upload what the host assigned since the last solve (stream-ordered).
int fd_upload(FDGrid* g, cudaStream_t s);
// One Solve on the device (fdtd.cpp:605-668), on stream s.
int fd_solve(FDGrid* g, cudaStream_t s);
// The solve of the coupled step: reads dA[1] (the cell vector as the
// coupling left it), writes dA[0].
cudaError_t fd_solve_coupled(const FDDev& p, const double* T, double* A, cudaStream_t s);
// sync_data (fdtd.cpp:599-603): the kept source, conductivity and capacity
// strings re-applied at the current step.
int fd_sync_data(FDGrid* g);
FDDev fd_dev(const FDGrid* g);

}  // namespace omdg

struct omdg_fdtd : omdg::FDGrid {};
