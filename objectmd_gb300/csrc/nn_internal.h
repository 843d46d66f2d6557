// Internal types of the atom-centred neural surrogate (no reference
// counterpart): descriptor parameters, the flat FP32 parameter vector, the
// model file, and the device image of the network for the tensor-core kernel.
#pragma once

#include <cuda_bf16.h>

#include <string>
#include <vector>

#include "omdg_internal.h"

namespace omdg {

constexpr int NN_RAD = 16;
constexpr int NN_ANG = 16;
constexpr int NN_DESC = NN_RAD + NN_ANG;  // 32 descriptors per atom
constexpr int NN_H = 64;                  // two hidden layers of 64
constexpr int NN_MAXN = 24;               // neighbours inside the descriptor cutoff one atom can hold

// flat parameter vector: W1[64x32] b1[64] W2[64x64] b2[64] w3[64] b3
constexpr int NN_OFF_W1 = 0;
constexpr int NN_OFF_B1 = NN_OFF_W1 + NN_H * NN_DESC;
constexpr int NN_OFF_W2 = NN_OFF_B1 + NN_H;
constexpr int NN_OFF_B2 = NN_OFF_W2 + NN_H * NN_H;
constexpr int NN_OFF_W3 = NN_OFF_B2 + NN_H;
constexpr int NN_OFF_B3 = NN_OFF_W3 + NN_H;
constexpr int NN_PARAMS = NN_OFF_B3 + 1;  // 6337

// Descriptor set and normalisation, passed to kernels by value.
//   radial  G_k = sum_j exp(-eta_r[k] (r - rs[k])^2) fc(r)
//   angular G_m = pref[m] sum_{j<k} (1 + lam[m] cos)^zeta[m] exp(-eta_a[m] (r_ij^2 + r_ik^2)) fc(r_ij) fc(r_ik)
//   fc(r) = 1 for r <= rin, (cos(pi (r - rin) / (rc - rin)) + 1) / 2 on (rin, rc)
// (rin = R - D, rc = R + D is Tersoff's own cutoff switch, tersoff.h:183)
struct NNDescParams {
    float rs[NN_RAD], eta_r[NN_RAD];
    float lam[NN_ANG], eta_a[NN_ANG], pref[NN_ANG];
    int zeta[NN_ANG];
    float rc, pi_rc;                       // pi_rc = pi / (rc - rin)
    float mu[NN_DESC], isig[NN_DESC];      // normalised input (G - mu) * isig
    float gmin[NN_DESC], gmax[NN_DESC];    // training range (fallback outside it)
    float rin;                             // inner radius of the cutoff switch (0: cosine over [0, rc])
};

struct NNModel {
    NNDescParams dp{};
    float sigma[NN_DESC] = {};
    std::vector<float> w;  // NN_PARAMS
};

// The default descriptor set: 16 radial centres on [1.6, 3.2] A with
// eta = 1 / (2 h^2) (h the spacing) and 16 angular terms
// (eta_a in {0, 0.3}) x (zeta in {1, 2, 4, 8}) x (lambda in {+1, -1}),
// cutoff rc = 3.2 A switched over [0, rc].
void nn_default_descriptors(NNDescParams& dp);
// Sets rc, rin and pi_rc; false unless 0 <= rin < rc.
bool nn_set_cutoff(NNDescParams& dp, float rc, float rin);
int nn_model_load(const std::string& path, NNModel& m, std::string& err);
int nn_model_save(const std::string& path, const NNModel& m, std::string& err);

// Device image of the network for k_nn_mlp: BF16 core-matrix tiles
// W1 [64x32], W2 [64x64], W2^T [64x64], W1^T [32x64] and FP32 vectors
// b1, b2, w3 (64 each), b3, and the input scale isig (32).
constexpr int NN_IMG_W1T = 0;                       // elements
constexpr int NN_IMG_W1 = NN_IMG_W1T + NN_DESC * NN_H;
constexpr int NN_IMG_W2 = NN_IMG_W1 + NN_H * NN_DESC;
constexpr int NN_IMG_W2T = NN_IMG_W2 + NN_H * NN_H;
constexpr int NN_IMG_ELEMS = NN_IMG_W2T + NN_H * NN_H;  // 12288 bf16 = 24 KB
constexpr int NN_VEC_B1 = 0, NN_VEC_B2 = 64, NN_VEC_W3 = 128, NN_VEC_B3 = 192, NN_VEC_ISIG = 196;
constexpr int NN_VEC_FLOATS = NN_VEC_ISIG + NN_DESC;  // 228

struct NNDevNet {
    __nv_bfloat16* img = nullptr;
    float* vec = nullptr;
};
int nn_net_upload(NNDevNet& net, const NNModel& m, cudaStream_t s, std::string& err);
void nn_net_free(NNDevNet& net);

// Tensor-core network over `rows` normalised descriptor rows: E (per row) and
// u = dE/dG in raw descriptor units (rows x 32).  Returns a cudaError.
cudaError_t nn_mlp_launch(const NNDevNet& net, const float* gt, int rows, float* E, float* u, unsigned* status,
                          int num_sms, cudaStream_t s);
// The same network with each row's descriptors computed in the kernel from
// the Verlet list (MD): flags atoms outside the training range and counts them.
// std_ang: the descriptor set has the default angular layout.
struct NNMD;
cudaError_t nn_mlp_md_launch(const NNDevNet& net, const NNMD& q, const NNDescParams& dp, bool std_ang,
                             const PosPack* pack, const unsigned* nbr, const int* nnb, int* flag, int* count,
                             float* E, float* u, unsigned* status, int num_sms, cudaStream_t s);

}  // namespace omdg
