// The finite-difference heat solver (FDTDSolver, src/omd/fdtd.cpp) on the
// device, single rank.
//
//   k_fd_solve   one thread per cell: the explicit step of Solve
//                (fdtd.cpp:605-668), reading the old cell vector and writing
//                the other buffer:
//                  acc = sum over exchange faces (r, l, b, t, n, f in that
//                        order) of K (T_nb - T_i), K = con_nb con_i / (con_nb + con_i)
//                  A_i = T_i + (2 acc / h^2 + S_i + E_i) dt / cap_i,  E_i = 0
//                A cell whose character is not in the symbol map skips the
//                face loop, so acc keeps its old value T_i (fdtd.cpp:607-610
//                copy A to T and leave A_i untouched) and the update reads it.
//
// The FP64 operations are the reference's, in its order, without
// contraction (explicit _rn intrinsics): results are bit-identical to the
// reference built with -ffp-contract=off.  A face's conductance
// K = con_a con_b / (con_a + con_b) is the same number seen from either cell
// (both operations commute), so k_fd_faces computes it once per face when
// the conductivity is uploaded and the step reads it: the step's FP64
// divisions drop from seven per cell to the one by cap.  The step then moves
// 8 B of the old vector, 24 B of its own three face conductances, 8 B cap,
// 8 B S, 8 B E, 4 B map and 1 B mask read and 8 B written per cell (69 B; E
// and S are cleared only where not zero); the neighbours' T and conductances
// come from L1/L2.  A face whose conductance is zero adds nothing, as in the
// reference for finite cell values.
//
// Host side (the string path of FDTDSolver, fdtd.cpp:100-118, 506-597): the
// symbol map, the map, and the assignment strings "<symbols> <value>[:t0[:t1]]"
// and "@ i,j,k[,i2,j2,k2]=<value>[:t0[:t1]]" with the reference's time-range
// pruning, applied to host images that are uploaded when they change.  A
// '{...}' value is an expression for muParser (a third-party library the
// reference does not vendor): it is refused with OMDG_EINVAL.
#include <cfloat>
#include <climits>
#include <cstring>
#include <sstream>

#include "fdtd_internal.h"

namespace omdg {

constexpr int FD_BLOCK = 256;

int fd_fail(FDGrid* g, int code, const std::string& msg) {
    g->err = msg;
    return code;
}

FDDev fd_dev(const FDGrid* g) {
    FDDev p;
    p.nx = g->nx;
    p.ny = g->ny;
    p.nz = g->nz;
    p.dim = g->dim;
    p.dt = g->timestep;
    p.h2inv = g->h2inv;
    p.map = g->dmap;
    p.mask = g->dmask[g->solves > 0 ? 1 : 0];
    p.K = g->dK;
    p.cap = g->dcap;
    p.S = g->dS;
    p.E = g->dE;
    p.mask_first = p.mask_later = nullptr;
    p.solves = p.active = nullptr;
    p.keep_S = 0;
    return p;
}

// The conductance of each cell's +x, +y and +z face (the neighbour wraps):
// K = con_nb con_i / (con_nb + con_i), 0 where con_nb + con_i is zero
// (fdtd.cpp:616-622).
__global__ void __launch_bounds__(FD_BLOCK) k_fd_faces(int nx, int ny, int nz, const double* __restrict__ con,
                                                       double* __restrict__ K) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int xy = nx * ny, dim = xy * nz;
    if (idx >= dim) return;
    const int k = idx / xy, a = idx % xy, j = a / nx, i = a % nx;
    const int nb[3] = {k * xy + (i + 1 == nx ? 0 : i + 1) + j * nx, k * xy + i + (j + 1 == ny ? 0 : j + 1) * nx,
                       (k + 1 == nz ? 0 : k + 1) * xy + i + j * nx};
    const double ci = con[idx];
    for (int d = 0; d < 3; d++) {
        const double cn = con[nb[d]];
        const double s = __dadd_rn(cn, ci);
        K[(size_t)d * dim + idx] = s != 0.0 ? __ddiv_rn(__dmul_rn(cn, ci), s) : 0.0;
    }
}

// K (T_nb - T_i) added to acc (fdtd.cpp:616-622)
__device__ __forceinline__ double fd_face(const double* __restrict__ T, double K, int nb, double ti, double acc) {
    if (K != 0.0) acc = __dadd_rn(acc, __dmul_rn(K, __dsub_rn(T[nb], ti)));
    return acc;
}

__global__ void __launch_bounds__(FD_BLOCK) k_fd_solve(FDDev p, const double* __restrict__ T, double* __restrict__ A) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= p.dim) return;
    if (p.active && !*p.active) return;  // coupled, model not active yet: the cell vector stays
    const double ti = T[idx];
    double acc = ti;  // a cell outside the symbol map keeps A_i = T_i
    if (p.map[idx] >= 0) {
        const int xy = p.nx * p.ny;
        const int k = idx / xy, a = idx % xy, j = a / p.nx, i = a % p.nx;
        const unsigned m = p.solves ? (*p.solves == 0 ? p.mask_first : p.mask_later)[idx] : p.mask[idx];
        const double* Kx = p.K;
        const double* Ky = p.K + p.dim;
        const double* Kz = p.K + 2 * (size_t)p.dim;
        acc = 0.0;
        // a face that is set and beyond the grid is periodic: it wraps (fdtd.cpp:277-285)
        if (m & FD_R) acc = fd_face(T, Kx[idx], k * xy + (i + 1 == p.nx ? 0 : i + 1) + j * p.nx, ti, acc);
        if (m & FD_L) {
            const int nb = k * xy + (i == 0 ? p.nx - 1 : i - 1) + j * p.nx;
            acc = fd_face(T, Kx[nb], nb, ti, acc);
        }
        if (m & FD_B) acc = fd_face(T, Ky[idx], k * xy + i + (j + 1 == p.ny ? 0 : j + 1) * p.nx, ti, acc);
        if (m & FD_T) {
            const int nb = k * xy + i + (j == 0 ? p.ny - 1 : j - 1) * p.nx;
            acc = fd_face(T, Ky[nb], nb, ti, acc);
        }
        if (p.nz != 1) {
            if (m & FD_N) {
                const int nb = (k == 0 ? p.nz - 1 : k - 1) * xy + i + j * p.nx;
                acc = fd_face(T, Kz[nb], nb, ti, acc);
            }
            if (m & FD_F) acc = fd_face(T, Kz[idx], (k + 1 == p.nz ? 0 : k + 1) * xy + i + j * p.nx, ti, acc);
        }
    }
    // A = T + (2 A h2inv + S + E) dt / cap (fdtd.cpp:664)
    const double si = p.S[idx], ei = p.E[idx];
    const double q = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0, acc), p.h2inv), si), ei);
    A[idx] = __dadd_rn(ti, __ddiv_rn(__dmul_rn(q, p.dt), p.cap[idx]));
    // E[i] = S[i] = 0 (fdtd.cpp:665), written only where not zero already
    if (ei != 0.0) p.E[idx] = 0.0;
    if (!p.keep_S && si != 0.0) p.S[idx] = 0.0;
}

int fd_solve(FDGrid* g, cudaStream_t s) {
    FDDev p = fd_dev(g);
    k_fd_solve<<<grid_for(g->dim, FD_BLOCK), FD_BLOCK, 0, s>>>(p, g->dA[g->cur], g->dA[g->cur ^ 1]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd solve: ") + cudaGetErrorString(e));
    g->cur ^= 1;
    g->solves += 1;
    return OMDG_OK;
}

cudaError_t fd_solve_coupled(const FDDev& p, const double* T, double* A, cudaStream_t s) {
    k_fd_solve<<<grid_for(p.dim, FD_BLOCK), FD_BLOCK, 0, s>>>(p, T, A);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ host: maps and strings
static int index3(const FDGrid* g, int i, int j, int k) { return (k * g->nx * g->ny) + (i + j * g->nx); }

static std::string replace_ch(std::string s, char a, char b) {
    for (char& c : s)
        if (c == a) c = b;
    return s;
}

static std::string remove_ch(const std::string& s, char d) {
    std::string r;
    for (char c : s)
        if (c != d) r += c;
    return r;
}

// as_double (omdtool.cpp:98-104): stream extraction, "inf" and "-inf" as +/-DBL_MAX
static bool to_double(const std::string& v, double& out) {
    if (v == "inf") {
        out = DBL_MAX;
        return true;
    }
    if (v == "-inf") {
        out = -DBL_MAX;
        return true;
    }
    std::istringstream ss(v);
    return (bool)(ss >> out);
}

// SetSymbolMap (fdtd.cpp:450-477)
static int parse_symbols(FDGrid* g, const std::string& str) {
    std::istringstream ss(str);
    while (ss.good()) {
        std::string tok, sb;
        if (!(ss >> tok >> sb)) break;
        if (sb.size() < 4) return fd_fail(g, OMDG_EINVAL, "invalid map symbol entry");
        auto flag = [](char c) { return c == '+' ? 1 : (c == 'p' ? 2 : 0); };
        for (char ch : tok) {
            FDBound b;
            b.sym = ch;
            b.l = flag(sb[0]);
            b.r = flag(sb[1]);
            b.t = flag(sb[2]);
            b.b = flag(sb[3]);
            if (g->nz > 1 && sb.size() == 6) {
                b.n = flag(sb[4]);
                b.f = flag(sb[5]);
            } else {
                b.n = b.f = 0;
            }
            g->bound.push_back(b);
        }
    }
    return OMDG_OK;
}

// The exchange directions each cell sees.  get_neigcell_index
// (fdtd.cpp:270-300) clears a symbol's flag for good when a cell of that
// symbol has the face beyond the grid and the flag is not periodic, so the
// first solve (cells visited in index order) and the later ones differ.
static void build_masks(FDGrid* g) {
    std::vector<FDBound> b = g->bound;
    g->mask_first.assign(g->dim, 0);
    for (int idx = 0; idx < g->dim; idx++) {
        if (g->map[idx] < 0) continue;
        const int xy = g->nx * g->ny, k = idx / xy, a = idx % xy, j = a / g->nx, i = a % g->nx;
        FDBound& c = b[g->map[idx]];
        if (i - 1 < 0 && c.l != 2) c.l = 0;
        if (i + 1 >= g->nx && c.r != 2) c.r = 0;
        if (j - 1 < 0 && c.t != 2) c.t = 0;
        if (j + 1 >= g->ny && c.b != 2) c.b = 0;
        if (g->nz != 1) {
            if (k - 1 < 0 && c.n != 2) c.n = 0;
            if (k + 1 >= g->nz && c.f != 2) c.f = 0;
        }
        g->mask_first[idx] = (c.r ? FD_R : 0) | (c.l ? FD_L : 0) | (c.b ? FD_B : 0) | (c.t ? FD_T : 0) |
                             (g->nz != 1 && c.n ? FD_N : 0) | (g->nz != 1 && c.f ? FD_F : 0);
    }
    g->mask_later.assign(g->dim, 0);
    for (int idx = 0; idx < g->dim; idx++) {
        if (g->map[idx] < 0) continue;
        const FDBound& c = b[g->map[idx]];  // the flags after one full pass; later passes change nothing
        g->mask_later[idx] = (c.r ? FD_R : 0) | (c.l ? FD_L : 0) | (c.b ? FD_B : 0) | (c.t ? FD_T : 0) |
                             (g->nz != 1 && c.n ? FD_N : 0) | (g->nz != 1 && c.f ? FD_F : 0);
    }
}

// check_expression (fdtd.cpp:100-118)
static void check_expression(std::string& str, int& t0, int& t1, bool& isequ) {
    isequ = str.find('{') != std::string::npos;
    std::istringstream sequ(remove_ch(remove_ch(replace_ch(str, ':', ' '), '{'), '}'));
    sequ >> str;
    if (sequ >> t0) {
        if (!(sequ >> t1)) t1 = t0;
    } else {
        t0 = -INT_MAX;
        t1 = INT_MAX;
    }
}

// AssignArray(ptr, str) (fdtd.cpp:528-592): tokens outside their time range
// are dropped from str, ranged ones in range are kept (an unranged token is
// kept for good).
static int assign_array(FDGrid* g, std::vector<double>& a, std::string& str, bool& changed) {
    if (str.empty()) return OMDG_OK;
    std::istringstream ss(str);
    str.clear();
    std::string tok, val;
    while (ss.good()) {
        if (!(ss >> tok >> val)) break;
        int t0, t1;
        bool isequ;
        check_expression(val, t0, t1, isequ);
        if (!(g->step >= t0 && g->step <= t1)) continue;
        if (t0 != t1) {
            if (isequ) str += tok + " {" + val + ":" + std::to_string(t0) + ":" + std::to_string(t1) + "} ";
            else str += tok + " " + val + ":" + std::to_string(t0) + ":" + std::to_string(t1) + " ";
        }
        if (isequ) return fd_fail(g, OMDG_EINVAL, "'{...}' expressions need muParser, which is not built: " + val);
        if (tok[0] == '@') {
            // coordinates before '=', the value after it (without '=' the
            // whole token is both, as val.erase(0, npos + 1) erases nothing)
            const size_t p = val.find('=');
            std::istringstream scor(replace_ch(val.substr(0, p), ',', ' '));
            const std::string v = p == std::string::npos ? val : val.substr(p + 1);
            int ix, iy, iz, jx, jy, jz;
            if (!(scor >> ix >> iy >> iz)) return fd_fail(g, OMDG_EINVAL, "wrong coordinate");
            auto put = [&](int i, int j, int k) -> int {
                const long long idx = (long long)k * g->nx * g->ny + i + (long long)j * g->nx;
                if (idx >= g->dim || idx < 0)
                    return fd_fail(g, OMDG_EINVAL,
                                   "AssignArray out of range: " + std::to_string(idx) + " (" + std::to_string(i) +
                                       "," + std::to_string(j) + "," + std::to_string(k) + ")");
                double dv;
                if (!to_double(v, dv)) return fd_fail(g, OMDG_EINVAL, "conversion error: " + v);
                if (!(a[idx] == dv) || std::signbit(a[idx]) != std::signbit(dv)) changed = true;
                a[idx] = dv;
                return OMDG_OK;
            };
            if (scor >> jx >> jy >> jz) {  // rectangle block
                if (g->nz == 1) iz = jz = 0;
                for (int i = ix; i <= jx; i++)
                    for (int j = iy; j <= jy; j++)
                        for (int k = iz; k <= jz; k++)
                            if (int rc = put(i, j, k)) return rc;
            } else if (int rc = put(ix, iy, iz)) {
                return rc;
            }
        } else {  // every cell whose symbol is in tok ('*' all, '.' cells outside the symbol map)
            double dv;
            const bool ok = to_double(val, dv);
            for (char c : tok)
                for (int i = 0; i < g->nx; i++)
                    for (int j = 0; j < g->ny; j++)
                        for (int k = 0; k < g->nz; k++) {
                            const int idx = index3(g, i, j, k);
                            const int m = g->map[idx];
                            const char sym = (m < 0 || m >= (int)g->bound.size()) ? '.' : g->bound[m].sym;
                            if (c == '*' || sym == c) {
                                if (!ok) return fd_fail(g, OMDG_EINVAL, "conversion error: " + val);
                                if (!(a[idx] == dv) || std::signbit(a[idx]) != std::signbit(dv)) changed = true;
                                a[idx] = dv;
                            }
                        }
        }
    }
    return OMDG_OK;
}

// assignments to S: the device S is zero after every solve, so any value
// written since makes the host image the one to upload
static int assign_source(FDGrid* g, std::string& str) {
    bool changed = false;
    const int rc = assign_array(g, g->hS, str, changed);
    if (changed) g->dirty_S = g->s_any = true;
    return rc;
}

int fd_sync_data(FDGrid* g) {
    bool ccon = false, ccap = false;
    int rc = assign_source(g, g->str_src);
    if (!rc) rc = assign_array(g, g->hcon, g->str_con, ccon);
    if (!rc) rc = assign_array(g, g->hcap, g->str_cap, ccap);
    g->dirty_con |= ccon;
    g->dirty_cap |= ccap;
    return rc;
}

// Host images that changed since the last upload go to the device
// (stream-ordered; the copy is staged before the call returns).
int fd_upload(FDGrid* g, cudaStream_t s) {
    const size_t b = sizeof(double) * g->dim;
    cudaError_t e = cudaSuccess;
    if (g->dirty_S) e = cudaMemcpyAsync(g->dS, g->hS.data(), b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && g->dirty_con) {
        e = cudaMemcpyAsync(g->dcon, g->hcon.data(), b, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
            k_fd_faces<<<grid_for(g->dim, FD_BLOCK), FD_BLOCK, 0, s>>>(g->nx, g->ny, g->nz, g->dcon, g->dK);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && g->dirty_cap) e = cudaMemcpyAsync(g->dcap, g->hcap.data(), b, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd upload: ") + cudaGetErrorString(e));
    g->dirty_S = g->dirty_con = g->dirty_cap = false;
    return OMDG_OK;
}

}  // namespace omdg

using namespace omdg;

static int fd_sync(omdg_fdtd* g) {
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd: ") + cudaGetErrorString(e));
    return OMDG_OK;
}

static int fd_download_A(omdg_fdtd* g) {
    cudaError_t e = cudaMemcpyAsync(g->hA.data(), g->dA[g->cur], sizeof(double) * g->dim, cudaMemcpyDeviceToHost,
                                    g->stream);
    if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd: ") + cudaGetErrorString(e));
    return fd_sync(g);
}

extern "C" {

int omdg_fdtd_create(omdg_fdtd** out, int device, int nx, int ny, int nz, const char* symbol, const char* map) {
    if (!out || !symbol || !map || nx < 1 || ny < 1 || nz < 1) return OMDG_EINVAL;
    *out = nullptr;
    if ((long long)nx * ny * nz > (1LL << 30)) return OMDG_EINVAL;
    omdg_fdtd* g = new omdg_fdtd();
    g->device = device;
    g->nx = nx;
    g->ny = ny;
    g->nz = nz <= 2 ? 1 : nz;  // nz <= 2: a 2D grid (fdtd.cpp:58-59)
    g->dim = g->nx * g->ny * g->nz;
    *out = g;
    int rc = parse_symbols(g, symbol);
    if (rc) return rc;
    if ((int)std::strlen(map) != g->dim) return fd_fail(g, OMDG_EINVAL, "map string count inconsistent");
    g->map.resize(g->dim);
    for (int i = 0; i < g->dim; i++) {  // search_symbol: the first entry with that character
        g->map[i] = -1;
        for (int b = 0; b < (int)g->bound.size(); b++)
            if (g->bound[b].sym == map[i]) {
                g->map[i] = b;
                break;
            }
    }
    build_masks(g);
    g->hA.assign(g->dim, 0.0);  // initiate_cells (fdtd.cpp:186-204)
    g->hS.assign(g->dim, 0.0);
    g->hcon.assign(g->dim, 1.0);
    g->hcap.assign(g->dim, 1.0);
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    g->own_stream = e == cudaSuccess;
    const size_t b8 = sizeof(double) * g->dim;
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = cudaMalloc(&g->dA[k], b8);
    if (e == cudaSuccess) e = cudaMalloc(&g->dS, b8);
    if (e == cudaSuccess) e = cudaMalloc(&g->dE, b8);
    if (e == cudaSuccess) e = cudaMalloc(&g->dcon, b8);
    if (e == cudaSuccess) e = cudaMalloc(&g->dK, 3 * b8);
    if (e == cudaSuccess) e = cudaMalloc(&g->dcap, b8);
    if (e == cudaSuccess) e = cudaMalloc(&g->dmap, sizeof(int) * g->dim);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = cudaMalloc(&g->dmask[k], g->dim);
    if (e != cudaSuccess) return fd_fail(g, OMDG_ENOMEM, std::string("fdtd allocation: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(g->dA[0], g->hA.data(), b8, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->dE, 0, b8, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->dmap, g->map.data(), sizeof(int) * g->dim, cudaMemcpyHostToDevice,
                                              g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->dmask[0], g->mask_first.data(), g->dim, cudaMemcpyHostToDevice,
                                              g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->dmask[1], g->mask_later.data(), g->dim, cudaMemcpyHostToDevice,
                                              g->stream);
    if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd: ") + cudaGetErrorString(e));
    if ((rc = fd_upload(g, g->stream))) return rc;
    return fd_sync(g);
}

int omdg_fdtd_destroy(omdg_fdtd* g) {
    if (!g) return OMDG_OK;
    if (g->coupled) return fd_fail(g, OMDG_ESTATE, "detach the grid from the two-temperature model first");
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (int k = 0; k < 2; k++) {
        cudaFree(g->dA[k]);
        cudaFree(g->dmask[k]);
    }
    cudaFree(g->dS);
    cudaFree(g->dE);
    cudaFree(g->dcon);
    cudaFree(g->dK);
    cudaFree(g->dcap);
    cudaFree(g->dmap);
    if (g->own_stream) cudaStreamDestroy(g->stream);
    delete g;
    return OMDG_OK;
}

const char* omdg_fdtd_last_error(omdg_fdtd* g) { return g ? g->err.c_str() : "null grid"; }

int omdg_fdtd_set_timestep(omdg_fdtd* g, double dt) {
    if (!g) return OMDG_EINVAL;
    g->timestep = dt;
    return OMDG_OK;
}

int omdg_fdtd_set_spacestep(omdg_fdtd* g, double h) {
    if (!g) return OMDG_EINVAL;
    g->spacestep = h;
    g->h2inv = 1.0 / (h * h);
    return OMDG_OK;
}

// which: 0 cell vector (SetCell), 1 source (SetSource), 2 conductivity, 3 capacity
int omdg_fdtd_assign(omdg_fdtd* g, int which, const char* str) {
    if (!g || !str || which < 0 || which > 3) return OMDG_EINVAL;
    if (g->coupled) return fd_fail(g, OMDG_ESTATE, "detach the grid from the two-temperature model first");
    cudaSetDevice(g->device);
    std::string s(str);
    int rc = OMDG_OK;
    if (which == 0) {
        if ((rc = fd_download_A(g))) return rc;
        bool changed = false;
        if ((rc = assign_array(g, g->hA, s, changed))) return rc;
        cudaError_t e = cudaMemcpyAsync(g->dA[g->cur], g->hA.data(), sizeof(double) * g->dim,
                                        cudaMemcpyHostToDevice, g->stream);
        if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd: ") + cudaGetErrorString(e));
        return fd_sync(g);
    }
    // SetSource / SetConductivity / SetCapacity keep the whole string and
    // apply a copy of it now (fdtd.hpp:126-133)
    std::string& kept = which == 1 ? g->str_src : (which == 2 ? g->str_con : g->str_cap);
    kept = str;
    if (which == 1) return assign_source(g, s);
    bool changed = false;
    rc = assign_array(g, which == 2 ? g->hcon : g->hcap, s, changed);
    if (which == 2) g->dirty_con |= changed;
    else g->dirty_cap |= changed;
    return rc;
}

// Step(n) (fdtd.cpp:671-689), single rank: per step sync_data, Solve, step++.
int omdg_fdtd_step(omdg_fdtd* g, int n) {
    if (!g || n < 0) return OMDG_EINVAL;
    if (g->coupled) return fd_fail(g, OMDG_ESTATE, "the grid is stepped by a context's two-temperature model");
    cudaSetDevice(g->device);
    for (int k = 0; k < n; k++) {
        int rc = fd_sync_data(g);
        if (!rc) rc = fd_upload(g, g->stream);
        if (!rc) rc = fd_solve(g, g->stream);
        if (rc) return rc;
        if (g->s_any) {  // Solve clears S (fdtd.cpp:665), on the device too
            std::fill(g->hS.begin(), g->hS.end(), 0.0);
            g->s_any = false;
        }
        g->step += 1;
    }
    return fd_sync(g);
}

// which: 0 cell vector, 1 source (as the next solve will see it), 2
// conductivity, 3 capacity, 4 external vector
int omdg_fdtd_get(omdg_fdtd* g, int which, double* out, long n) {
    if (!g || !out || n != g->dim || which < 0 || which > 4) return OMDG_EINVAL;
    cudaSetDevice(g->device);
    if (which == 0 || which == 4) {
        cudaError_t e = cudaMemcpyAsync(out, which == 0 ? g->dA[g->cur] : g->dE, sizeof(double) * n,
                                        cudaMemcpyDeviceToHost, g->stream);
        if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd: ") + cudaGetErrorString(e));
        return fd_sync(g);
    }
    const std::vector<double>& a = which == 1 ? g->hS : (which == 2 ? g->hcon : g->hcap);
    std::memcpy(out, a.data(), sizeof(double) * n);
    return OMDG_OK;
}

// GetExtVector() written by the caller: E for the next solve, which clears it.
int omdg_fdtd_set_ext(omdg_fdtd* g, const double* e_in, long n) {
    if (!g || !e_in || n != g->dim) return OMDG_EINVAL;
    if (g->coupled) return fd_fail(g, OMDG_ESTATE, "the coupling writes the external vector");
    cudaSetDevice(g->device);
    cudaError_t e = cudaMemcpyAsync(g->dE, e_in, sizeof(double) * n, cudaMemcpyHostToDevice, g->stream);
    if (e != cudaSuccess) return fd_fail(g, OMDG_ECUDA, std::string("fdtd: ") + cudaGetErrorString(e));
    return fd_sync(g);
}

int omdg_fdtd_info(omdg_fdtd* g, int* nx, int* ny, int* nz, int* step) {
    if (!g) return OMDG_EINVAL;
    if (nx) *nx = g->nx;
    if (ny) *ny = g->ny;
    if (nz) *nz = g->nz;
    if (step) *step = g->step;
    return OMDG_OK;
}

}  // extern "C"
