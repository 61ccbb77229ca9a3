// Per-sector dense decomposition tables and kernels (decomp.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "imps_internal.h"

namespace imps {

// One block of a block-sparse object copied into (or out of) a packed dense sector matrix.
struct GatherEntry {
  int64_t src_off;  // block offset in the block-sparse vector
  int64_t dst_off;  // offset of the dense matrix in the packed buffer
  int32_t rows, cols;
  int32_t r0, c0;   // position of the block inside the dense matrix
  int32_t dst_ld;
  int32_t transpose;  // 1: the dense matrix holds the transpose of the stacked blocks
};

// One dense sector matrix (M x N, "tall" orientation, M >= N expected).
struct DenseMat {
  int64_t a_off;  // packed M x N input / U output
  int64_t q_off;  // Q (M x K) / U (M x N)
  int64_t r_off;  // R (K x N) / V (N x N) / DiagIso
  int64_t s_off;  // singular values (N)
  int64_t w_off;  // scratch (N + M*N)
  int64_t ns_off; // null space (M x (M - N)), dir l only
  int32_t M, N;
};

struct DecompPlan {
  int dir = 0;
  std::vector<GatherEntry> ent;
  std::vector<DenseMat> mats;
  int64_t dense_elems = 0, r_elems = 0, s_elems = 0, w_elems = 0;
  bool tall = true;  // every sector has M >= N
  Layout rlayout;    // R / DiagIso BlockDiag layout over the sectors
  // left null space (dir l, Nullspace(A, l), MPSBlockUtilities.hpp:247-300): per physical
  // index s the blocks (Qin -> q) of A whose right sector q has M > N, with M - N columns
  Layout nslayout;
  std::vector<GatherEntry> nent;  // dense null-space rows -> N_L blocks
  int64_t ns_elems = 0;
  GatherEntry* d_nent = nullptr;
  double* dNS = nullptr;
  GatherEntry* d_ent = nullptr;
  DenseMat* d_mats = nullptr;
  double* dA = nullptr;  // dense input (overwritten by QR / holds U for SVD)
  double* dQ = nullptr;  // dense Q
  double* dR = nullptr;  // R or V
  double* dV2 = nullptr; // V^T (DiagIso for dir l)
  double* dS = nullptr;
  double* dW = nullptr;
  int* dstatus = nullptr;
};

int build_decomp(DecompPlan& D, const Layout& A, int dir);

int dc_gather(const GatherEntry* d_ent, int nent, const double* src, double* dense, cudaStream_t st);
int dc_scatter(const GatherEntry* d_ent, int nent, const double* dense, double* dst, cudaStream_t st);
int dc_qr(const DenseMat* d_mats, int nmat, double* A, double* Q, double* R, int transpose_r, cudaStream_t st);
// Largest sector dimension N handled by the shared-memory SVD (R and V, N x N each, in shared
// memory); larger sectors use the global-memory Jacobi kernel.
constexpr int kJacobiMaxN = 118;
// Largest N of the mixed-precision SVD (R, V and an FP32 / scratch square in shared memory).
constexpr int kMixedMaxN = 96;
int dc_svd(const DenseMat* d_mats, int nmat, int maxN, int64_t maxMN, double* U, double* S, double* V, double* W,
           int* status, cudaStream_t st);
// Up to kSvdSets independent sector SVDs (e.g. the two polar steps of a site update) in one
// launch: set k's sectors are CTAs [sum_{j<k} n_j, sum_{j<=k} n_j).
constexpr int kSvdSets = 4;
struct SvdSet {
  const DenseMat* mats;
  double *U, *S, *V, *W;
  int n;
};
struct SvdSets {
  SvdSet s[kSvdSets];
  int nsets;
};
int dc_svd_sets(const SvdSets& sets, int maxN, int64_t maxMN, int* status, cudaStream_t st);
int dc_colscale(const DenseMat* d_mats, int nmat, double* X, const double* S, double power, cudaStream_t st);
int dc_transpose_sq(const DenseMat* d_mats, int nmat, const double* X, double* Y, cudaStream_t st);
int dc_nullspace(const DenseMat* d_mats, int nmat, double* A, double* NS, cudaStream_t st);

}  // namespace imps
