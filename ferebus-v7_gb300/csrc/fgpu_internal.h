// Internal declarations shared by the engine's translation units.
//
// Data layout in HBM (one problem = one training set evaluated at one theta):
//
//   planes  : nplanes x Nc doubles, plane-major.  One plane per (leaf, active
//             dim): x for rbf / rbf-cyclic / linear, and the pair
//             sin(x/2), cos(x/2) for periodic, so that
//             sin((xi-xj)/2) = s_i c_j - c_i s_j needs no FP64 sin per pair.
//   K       : ld x Nc, column-major (Fortran order, like the reference's
//             covariance_matrix).  Nc = N rounded up to TB; ld = Nc + TB.
//             Rows [0, N) x cols [0, N): k(X, X) + nugget (lower triangle).
//             Rows/cols [N, Nc): identity padding, so every panel is full.
//             Rows [Nc, Nc + nrhs): the right-hand sides r_q^T (border rows);
//             the Cholesky sweep turns them into (L^-1 r_q)^T, which is all
//             the log-likelihood needs.  Rows [Nc + nrhs, ld): zero.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

namespace fgpu {

constexpr int TB = 64;            // panel width and tile edge
constexpr int MAX_LEAF = 8;
constexpr int MAX_POST = 16;
constexpr int MAX_PLANES = 192;
constexpr int MAX_PARAMS = 256;
constexpr int MAX_RHS = 2;

enum LeafType { L_RBF = 1, L_PERIODIC = 2, L_RBF_CYCLIC = 3, L_LINEAR = 4, L_CONSTANT = 5 };
enum PostTok : int8_t { P_SUM = -1, P_PROD = -2 };

struct Leaf {
  int type;     // LeafType
  int n;        // active dims (0 for constant)
  int plane0;   // first plane of this leaf
  int param0;   // first kernel parameter of this leaf
};

struct Spec {
  int nleaf;
  Leaf leaf[MAX_LEAF];
  int npost;
  int8_t post[MAX_POST];          // >= 0: leaf index; P_SUM / P_PROD
  int nplanes;
  int nkparams;
  uint8_t cyclic[MAX_PLANES];     // rbf-cyclic: plane's feature index is 3, 6, 9, ... (1-based)
  // tensor-core build (tensor-core mode; leaves rbf / periodic / linear /
  // constant, at most 2 rbf or periodic "distance" leaves, <= 128 digit columns)
  int tc_build;
  int ndot;                       // distance leaves
  int dot_leaf[2];                // their leaf indices
  int dot_koff[2];                // first digit column (multiple of 16)
  int dot_kch[2];                 // k chunks of 16
  int dot_u[2];                   // W units: <f_i, f_j> 2^(u - 2 - 2s)
};

// Per-problem descriptor, resident in device memory.
struct Prob {
  int N, Nc, ld, nsteps, nrhs, likelihood, optimise_noise, nkparams;
  double noise;
  const double* planes;           // nplanes x Nc
  const double* y;                // Nc, zero padded
  const double* mu;               // Nc, zero padded (marginal)
  const Spec* spec;
  const double* theta;            // raw parameters
  double* K;                      // ld x Nc
  double* logdet_part;            // nsteps
  int* status;                    // [0] info (LAPACK convention), [1] failed flag
  double* out;                    // [0] ll, [1] logdet, [2] mean, [3] sigma2
  double* z;                      // Nc: the vector alpha's back-substitution starts from
  double* ll_dst;                 // optional extra destination for ll (batch output)
  int* info_dst;                  // optional extra destination for info
  // tensor-core (split-integer) trailing update; unused in FP64 mode
  int mode;                       // 0: FP64 mma.sync 64-panels, 1: tcgen05 split update, 128-panels
  int nt128;                      // Nc / 128 (mode 1)
  int* escale;                    // Nc: per-row power-of-two scale e_i, |L_ik| <= 2^e_i
  double* pw2;                    // Nc: 2^(e_i - 31)
  long long* acc;                 // lower-triangle 128 x 64 tiles: exact sums of products W, value
                                  // W 2^(e_i + e_j - 62); |W| < 2^62 (Cauchy-Schwarz with the row scales)
  unsigned char* slices;          // nt128 x 7 x 32 KB: fp16 digit planes of the current panel
  const void* tmap_a;             // TMA tensor map over slices, box 8 x 128 rows x 2 kgroups x 7 planes
  const void* tmap_b;             // same, box of 64 rows
  const void* tmap_bs;            // box of 64 rows landing as [k-group][plane][row]: the 7 planes stacked along N
  const void* tmap_bs32;          // same, box of 32 rows
  // dot-product kernel build (mode 1): planes scaled by sqrt(l_k) per evaluation
  double* splanes;                // nplanes x Nc
  double* norms;                  // MAX_LEAF x Nc: sum_k u_ik^2 of rbf leaves
  // FP64 kernels: number of 64-row tiles when extra border rows follow the
  // right-hand-side tile (the adjoint's identity rows); 0 = nsteps + 1
  int nrt;
  // adjoint on a tensor-core context: K already holds the final factor L
  // (from the tensor-core evaluation), so the FP64 sweep works only on the
  // identity rows below the right-hand-side tile
  int border_only;
  double* kinv;                   // adjoint: K^-1 (Nc x Nc, lower)
  double* gpart;                  // adjoint: per-CTA partial sums
  // tensor-core build
  const double* plane_max;        // nplanes: max_i |planes[p][i]|
  long long* fnorm;               // 2 x Nc: W_ii of the distance leaves
  double* fcoef;                  // 4: k = a + b v0 + c v1 + d v0 v1
  int* fscale;                    // 2: s of the distance leaves, max |f| < 2^s
};

// Encode the four 5-D TMA tensor maps of a problem's digit-plane buffer
// (boxes of 128 and 64 rows, and 64 and 32 rows with the planes stacked)
// into host memory (4 x 128 bytes).  Returns 0 or a CUDA driver error code.
int encode_slice_maps(void* host_maps, const void* slices, int nt128);

// Launch helpers (engine.cu).  All kernels take a device array of problems
// and index it by blockIdx.y; problems whose geometry does not reach the
// current step exit immediately, so ragged batches share one launch.
cudaError_t launch_build(const Prob* probs, int nprob, int max_nsteps, int max_nplanes, cudaStream_t s);
// mode 1: per-evaluation scaled planes, then the dot-product form of the build
cudaError_t launch_prep_planes(const Prob* probs, int nprob, int max_nc, cudaStream_t s);
cudaError_t launch_build_dot(const Prob* probs, int nprob, int max_nsteps, int max_nplanes, cudaStream_t s);
size_t build_dot_smem_bytes(int nplanes);
cudaError_t launch_potf2(const Prob* probs, int nprob, int step, cudaStream_t s);
// tensor-core mode: the 32 x 32 diagonal block of quarter q of panel step, and
// the rows below it up to max_rows (the tallest problem's ld), which also
// writes their fp16 digit planes
constexpr int QW = 32;
cudaError_t launch_potf2_quarter(const Prob* probs, int nprob, int step, int q, cudaStream_t s);
// quarter panel solve (ozaki.cu): FP64 substitution in two 16-column halves coupled on the tensor cores
cudaError_t launch_trsm_quarter(const Prob* probs, int nprob, int step, int q, int max_rows, cudaStream_t s);
// max_rowtiles: 64-row tiles of the tallest problem (0 = max_nsteps + 1)
cudaError_t launch_trsm(const Prob* probs, int nprob, int step, int max_nsteps, cudaStream_t s,
                        int max_rowtiles = 0);
cudaError_t launch_update(const Prob* probs, int nprob, int step, int max_nsteps, cudaStream_t s,
                          int max_rowtiles = 0);
cudaError_t launch_finalize(const Prob* probs, int nprob, cudaStream_t s);
cudaError_t launch_backsolve(const Prob* probs, int nprob, int max_nsteps, double* alpha_out,
                             cudaStream_t s, long long* nlaunch);
size_t build_smem_bytes(int nplanes);

// Split-integer tensor-core path (ozaki.cu): 128-wide panels.
constexpr int NB = 128;
constexpr int NSLICE = 7;                       // fp16 digit planes per FP64 value
constexpr size_t SLICE_BYTES = 128 * 128 * 2;   // one digit plane of a 128-row x 128-k tile
// The exact trailing sums are kept for lower-triangle tiles only (128 rows x
// 64 columns), one int64 per element: column tile tj holds row tiles tj / 2
// .. nt128 - 1, so a problem stores nt128 (nt128 + 1) tiles instead of
// (2 nt128) nt128.  acc_tile is the tile's index in that packed order.
// Inside a tile the elements are grouped in 32 pieces of 2 KB, one per
// (8-column group, 32-row quarter), each column-major (8 columns x 32 rows):
// the piece one epilogue warp of the trailing update adds in a single bulk
// reduction.  acc_elem is an element's index inside its tile.
__host__ __device__ inline size_t acc_tile(int ti, int tj, int nt128) {
  const long long q = tj >> 1, h = tj & 1;
  return (size_t)(2 * q * nt128 - q * (q - 1) + h * (nt128 - q) + (ti - q));
}
inline size_t acc_tiles(int nt128) { return (size_t)nt128 * (nt128 + 1); }
__host__ __device__ inline int acc_elem(int r, int c) {  // row r < 128, column c < 64 of the tile
  return (((c >> 3) * 4 + (r >> 5)) << 8) + ((c & 7) << 5) + (r & 31);
}
constexpr size_t ACC_TILE_ELEMS = (size_t)NB * TB;

cudaError_t launch_scales(const Prob* probs, int nprob, int max_nc, cudaStream_t s);
cudaError_t launch_panel_prep(const Prob* probs, int nprob, int step, int max_nc, cudaStream_t s);
// prefix: device table of nprob + 1 tile offsets for this step (tiles of
// problem p at step s: m (m + 1), m = nt128_p - s - 1); total_tiles = prefix[nprob].
// tiles: the step's trailing tiles, packed (problem << 40 | row tile << 20 | column tile)
cudaError_t launch_ozaki_update(const Prob* probs, int nprob, int step, int max_nt128,
                                const unsigned long long* tiles, int total_tiles, int num_sms, cudaStream_t s);
cudaError_t launch_border_update(const Prob* probs, int nprob, int step, int max_nc, cudaStream_t s);
// four 32-column quarters per 128-panel (their digit planes are written by
// the quarter panel solve): the tensor-core coupling of source quarters
// [sq, sq + ns) into destination quarters [dq, dq + nq), nq = 1 or 2 (with
// the right-hand-side rows in FP64), which also factors quarter dq's
// diagonal block.  order: the step's total_tiles row tiles as
// (problem << 16 | ti), each problem's own row tile first; counter: a zeroed
// int the CTAs take tiles from.
cudaError_t launch_couple(const Prob* probs, int nprob, int step, int sq, int ns, int dq, int nq,
                          const int* order, int total_tiles, int* counter, int num_sms, cudaStream_t s);

// Tensor-core kernel-matrix build (build_tc.cu): feature digit planes and
// exact self products, then the persistent build of the lower triangle.
// tiles: the lower triangle's 128 x 64 tiles of every eligible problem,
// packed (problem << 40 | row tile << 20 | column tile).
cudaError_t launch_feat_digits(const Prob* probs, int nprob, int max_nt128, cudaStream_t s);
cudaError_t launch_build_tc(const Prob* probs, int nprob, const unsigned long long* tiles, int total_tiles,
                            int num_sms, cudaStream_t s);

// Adjoint (grad.cu): identity rows below the right-hand-side tile turn into
// L^-T during the sweep; K^-1 = L^-T (L^-T)^T; fused dK/dtheta pass.
cudaError_t launch_identity_border(const Prob* p, int nc, cudaStream_t s);
cudaError_t launch_syrk_inv(const Prob* p, int nsteps, cudaStream_t s);
cudaError_t enqueue_grad_passes(const Prob* p, int nsteps, int nk, int optimise_noise, double* g_out,
                                cudaStream_t s, long long* nlaunch);
constexpr int GRAD_SLOTS = 33;  // parameters per fused pass + noise slot

// Opt kernel `func` into `bytes` of dynamic shared memory on the CURRENT
// device.  cudaFuncSetAttribute acts per device, so the record of what was
// already set is one bit per (device, slot), updated atomically: a second
// device, or a second thread, sets the attribute for itself.  Devices
// beyond the first 64 set it on every call.
enum SmemSlot {
  SMEM_BUILD, SMEM_BUILD_DOT, SMEM_UPDATE, SMEM_SYRK, SMEM_OZAKI_UPDATE, SMEM_COUPLE1, SMEM_COUPLE2,
  SMEM_BUILD_TC, SMEM_NSLOTS
};
cudaError_t ensure_smem_attr(const void* func, int slot, int bytes);

// api.cu hooks for other translation units.
int internal_compile_spec(const int* kspec, int nkspec, int d, Spec& sp, std::vector<int>& plane_dim,
                          std::vector<int>& plane_kind);
int internal_fail(int code, const char* msg);
void internal_clear_error();
void internal_add_launches(long long n);

}  // namespace fgpu
