// FP64 engine kernels: kernel-matrix build, blocked right-looking Cholesky
// (diagonal factor, panel solve, trailing update on the FP64 MMA pipe),
// likelihood epilogue and the back-substitution for alpha.
//
// Every kernel takes the device array of problem descriptors and indexes it
// by blockIdx.z (tile kernels) or blockIdx.x (per-problem kernels), so one
// launch serves a whole ragged batch.
#include "../../include/fgpu.h"
#include "fgpu_internal.h"
#include "iexp.cuh"
#include "tc_common.cuh"
#include "potf2_block.cuh"

#include <atomic>
#include <cmath>
#include <cstdio>

namespace fgpu {

#define FGPU_PI 3.141592653589793115997963468544185161590576171875
#define FGPU_TWOPI 6.28318530717958623199592693708837032318115234375
#define FGPU_LOG_TWOPI 1.8378770664093453390819377091247588396072387695312

// ---------------------------------------------------------------------------
// kernel-matrix build
// ---------------------------------------------------------------------------
// Raw parameters -> stored kernel parameters (rbf_kernel.f90:113-119,
// periodic_kernel.f90:111-118, rbf_cyclic_kernel.f90:109-115,
// linear_kernel.f90:94-100, constant.f90:86-90).
__device__ __forceinline__ double transform_param(int type, double t) {
  switch (type) {
    case L_RBF:
    case L_RBF_CYCLIC:
      return exp(t);
    case L_PERIODIC: {
      double l = 1.0 / exp(t);
      return l * l;
    }
    case L_LINEAR:
      return exp(-t);
    default:
      return t;
  }
}

// One leaf at one (i, j) pair.  Pi / Pj point at the row / column tile's
// planes in shared memory (plane p of point r at P[p * TB + r]).
__device__ __forceinline__ double leaf_value(const Leaf& L, const double* __restrict__ Pi,
                                             const double* __restrict__ Pj, int ri, int cj,
                                             const double* __restrict__ ls, const uint8_t* cyc,
                                             double lin_sum) {
  const int p0 = L.plane0, q0 = L.param0, n = L.n;
  switch (L.type) {
    case L_RBF: {
      // stationary_kernel.f90:101-122: exp(-0.5 * sum_k l_k (x_ik - x_jk)^2)
      double acc = 0.0;
      for (int k = 0; k < n; ++k) {
        double dlt = Pi[(p0 + k) * TB + ri] - Pj[(p0 + k) * TB + cj];
        acc = fma(ls[q0 + k], dlt * dlt, acc);
      }
      return iexp_neg(-0.5 * acc);
    }
    case L_PERIODIC: {
      // periodic_kernel.f90:181-206 on distance_matrix.f90:130-142:
      // exp(-2 * sum_k l_k sin^2(|x_ik - x_jk| / 2)), with
      // sin((a-b)/2) = sin(a/2)cos(b/2) - cos(a/2)sin(b/2).
      double acc = 0.0;
      for (int k = 0; k < n; ++k) {
        const double si = Pi[(p0 + 2 * k) * TB + ri], ci = Pi[(p0 + 2 * k + 1) * TB + ri];
        const double sj = Pj[(p0 + 2 * k) * TB + cj], cjv = Pj[(p0 + 2 * k + 1) * TB + cj];
        double t = fma(si, cjv, -(ci * sj));
        acc = fma(ls[q0 + k], t * t, acc);
      }
      return iexp_neg(-2.0 * acc);
    }
    case L_RBF_CYCLIC: {
      // stationary_cyclic_kernel.f90:104-127 on distance_matrix.f90:95-128:
      // every 3rd feature's difference wrapped to [-pi, pi].
      double acc = 0.0;
      for (int k = 0; k < n; ++k) {
        double dlt = Pi[(p0 + k) * TB + ri] - Pj[(p0 + k) * TB + cj];
        if (cyc[p0 + k]) {
          double a = fabs(dlt) + FGPU_PI;
          dlt = copysign(1.0, dlt) * (fmod(a, FGPU_TWOPI) - FGPU_PI);
        }
        acc = fma(ls[q0 + k], dlt * dlt, acc);
      }
      return iexp_neg(-0.5 * acc);
    }
    case L_LINEAR:
      // linear_kernel.f90:70-76 with the reference's default order 0:
      // sum_k (x_ik x_jk)^0 / c_k, independent of (i, j).
      return lin_sum;
    default:
      return ls[q0];  // constant.f90:62-68
  }
}

__device__ __forceinline__ double kernel_value(const Spec& sp, const double* Pi, const double* Pj, int ri,
                                               int cj, const double* ls, const double* lin_sums) {
  double stk[MAX_LEAF];
  int top = 0;
  for (int t = 0; t < sp.npost; ++t) {
    const int tok = sp.post[t];
    if (tok >= 0) {
      stk[top++] = leaf_value(sp.leaf[tok], Pi, Pj, ri, cj, ls, sp.cyclic, lin_sums[tok]);
    } else {
      const double b = stk[--top];
      const double a = stk[--top];
      stk[top++] = (tok == P_SUM) ? a + b : a * b;  // kernel_module.f90:309-325 / 359-375
    }
  }
  return stk[0];
}

size_t build_smem_bytes(int nplanes) {
  return (size_t)2 * nplanes * TB * sizeof(double) + 64;
}

// grid: (row tile 0..nsteps, col tile 0..nsteps-1, problem); 256 threads.
// Each thread produces 2 consecutive rows x 8 columns of the 64 x 64 tile and
// writes them as double2 so that a warp stores 512 contiguous bytes.
__global__ void __launch_bounds__(256) k_build(const Prob* __restrict__ probs) {
  const Prob& P = probs[blockIdx.z];
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (tj >= P.nsteps || ti > P.nsteps || ti < tj) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const Spec& sp = *P.spec;
  const int np = sp.nplanes;
  double* Pi = reinterpret_cast<double*>(smem_raw);
  double* Pj = Pi + (size_t)np * TB;
  uint64_t* bar = reinterpret_cast<uint64_t*>(Pj + (size_t)np * TB);
  __shared__ double ls[MAX_PARAMS];
  __shared__ double lin_sums[MAX_LEAF];
  __shared__ int s_fail;

  const int tid = threadIdx.x;
  const bool border = (ti == P.nsteps);
  const int i0 = ti * TB, j0 = tj * TB;

  if (tid == 0) {
    s_fail = 0;
    if (np > 0) {
      mbar_init(bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
  }
  __syncthreads();
  if (tid == 0 && np > 0) {
    const uint32_t per = TB * sizeof(double);
    const uint32_t total = per * np * (border ? 1 : 2);
    mbar_expect_tx(bar, total);
    for (int p = 0; p < np; ++p) {
      bulk_g2s(Pj + p * TB, P.planes + (size_t)p * P.Nc + j0, per, bar);
      if (!border) bulk_g2s(Pi + p * TB, P.planes + (size_t)p * P.Nc + i0, per, bar);
    }
  }
  // parameters while the copies fly
  for (int k = tid; k < sp.nkparams; k += blockDim.x) {
    int type = L_CONSTANT;
    for (int l = 0; l < sp.nleaf; ++l) {
      const int cnt = sp.leaf[l].type == L_CONSTANT ? 1 : sp.leaf[l].n;
      if (k >= sp.leaf[l].param0 && k < sp.leaf[l].param0 + cnt) type = sp.leaf[l].type;
    }
    ls[k] = transform_param(type, P.theta[k]);
  }
  __syncthreads();
  if (tid < sp.nleaf) {
    double s = 0.0;
    const Leaf& L = sp.leaf[tid];
    if (L.type == L_LINEAR)
      for (int k = 0; k < L.n; ++k) s += 1.0 / ls[L.param0 + k];
    lin_sums[tid] = s;
  }
  if (np > 0 && !mbar_wait(bar, 0)) s_fail = 1;
  __syncthreads();
  if (s_fail) {
    // copy engine did not answer: report, do not hang; the copies land
    // (bounded wait) before the block's shared memory is released
    if (tid == 0) {
      mbar_wait(bar, 0);
      atomicExch(&P.status[2], 1);
    }
    return;
  }

  const double noise = P.optimise_noise ? P.theta[sp.nkparams] : P.noise;
  const int r0 = (tid & 31) * 2;
  const int c0 = (tid >> 5) * 8;
  double* K = P.K;
  const size_t ld = (size_t)P.ld;
  for (int cc = 0; cc < 8; ++cc) {
    const int c = c0 + cc, j = j0 + c;
    double v[2];
    for (int a = 0; a < 2; ++a) {
      const int r = r0 + a, i = i0 + r;
      double val = 0.0;
      if (border) {
        const int q = r;
        if (j < P.N && q < P.nrhs) {
          if (q == 0)
            val = (P.likelihood == 1) ? P.y[j] : P.y[j] - P.mu[j];
          else
            val = 1.0;
        }
      } else if (i < P.N && j < P.N) {
        if (i >= j) {
          val = kernel_value(sp, Pi, Pj, r, c, ls, lin_sums);
          if (i == j) val = val + noise * 1.0;  // gpr.f90:188, nugget * identity
        }
      } else {
        val = (i == j) ? 1.0 : 0.0;  // identity padding
      }
      v[a] = val;
    }
    *reinterpret_cast<double2*>(K + (size_t)j * ld + i0 + r0) = make_double2(v[0], v[1]);
  }
}

// ---------------------------------------------------------------------------
// dot-product form of the kernel-matrix build (tensor-core mode)
//
// With u_ik = sqrt(l_k) (x_ik - xbar_k) and a_i = sum_k u_ik^2,
//   sum_k l_k (x_ik - x_jk)^2 = a_i + a_j - 2 <u_i, u_j>,
// and with v_ik = sqrt(l_k) (cos x_ik, sin x_ik),
//   2 sum_k l_k sin^2((x_ik - x_jk) / 2) = sum_k l_k - <v_i, v_j>,
// so an rbf or periodic leaf costs one FP64 FMA per feature and pair instead
// of three or four.  The rounding error of the exponent is about u * a_i
// (absolute) on centred features, the size of its own rounding in the direct
// form for the well separated pairs that dominate, and it vanishes on the
// diagonal, which is set exactly (x_i = x_j gives a factor 1).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_prep_planes(const Prob* __restrict__ probs) {
  const Prob& P = probs[blockIdx.z];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (P.mode != 1 || i >= P.Nc) return;
  const Spec& sp = *P.spec;
  const size_t nc = (size_t)P.Nc;
  // the workspace is not cleared between evaluations (a batch plan reuses
  // it across problems): rows of non-rbf leaves are zeroed here
  if (l >= sp.nleaf || sp.leaf[l].type != L_RBF) P.norms[(size_t)l * nc + i] = 0.0;
  if (l >= sp.nleaf) return;
  const Leaf& L = sp.leaf[l];
  if (L.type == L_RBF) {
    double a = 0.0;
    for (int k = 0; k < L.n; ++k) {
      const double w = exp(0.5 * P.theta[L.param0 + k]);  // sqrt(exp(theta))
      const double u = w * P.planes[(size_t)(L.plane0 + k) * nc + i];
      P.splanes[(size_t)(L.plane0 + k) * nc + i] = u;
      a = fma(u, u, a);
    }
    P.norms[(size_t)l * nc + i] = a;
  } else if (L.type == L_PERIODIC) {
    for (int k = 0; k < L.n; ++k) {
      const double w = 1.0 / exp(P.theta[L.param0 + k]);  // sqrt((1 / exp(theta))^2)
      for (int t = 0; t < 2; ++t) {
        const size_t o = (size_t)(L.plane0 + 2 * k + t) * nc + i;
        P.splanes[o] = w * P.planes[o];
      }
    }
  } else if (L.type == L_RBF_CYCLIC) {
    for (int k = 0; k < L.n; ++k) {
      const size_t o = (size_t)(L.plane0 + k) * nc + i;
      P.splanes[o] = P.planes[o];
    }
  }
}

size_t build_dot_smem_bytes(int nplanes) {
  return (size_t)2 * (nplanes + MAX_LEAF) * TB * sizeof(double) + 64;
}

__global__ void __launch_bounds__(256) k_build_dot(const Prob* __restrict__ probs) {
  const Prob& P = probs[blockIdx.z];
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (P.mode != 1 || tj >= P.nsteps || ti > P.nsteps || ti < tj) return;
  const Spec& sp = *P.spec;
  if (sp.tc_build && ti != P.nsteps) return;  // built on the tensor cores; only its RHS rows here
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int np = sp.nplanes;
  const int nl = sp.nleaf;
  double* Pi = reinterpret_cast<double*>(smem_raw);      // np x 64 planes, row points
  double* Pj = Pi + (size_t)np * TB;                      // column points
  double* Ni = Pj + (size_t)np * TB;                      // nl x 64 norms, row points
  double* Nj = Ni + (size_t)MAX_LEAF * TB;
  uint64_t* bar = reinterpret_cast<uint64_t*>(Nj + (size_t)MAX_LEAF * TB);
  __shared__ double ls[MAX_PARAMS];
  __shared__ double leaf_c[MAX_LEAF];  // sum of l (periodic) or sum of 1/c (linear)
  __shared__ int s_fail;
  const int tid = threadIdx.x;
  const bool border = (ti == P.nsteps);
  const int i0 = ti * TB, j0 = tj * TB;
  const size_t nc = (size_t)P.Nc;
  if (tid == 0) {
    s_fail = 0;
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t per = TB * sizeof(double);
    const uint32_t nrows = (uint32_t)(np + nl);
    mbar_expect_tx(bar, per * nrows * (border ? 1 : 2));
    for (int p = 0; p < np; ++p) {
      bulk_g2s(Pj + p * TB, P.splanes + (size_t)p * nc + j0, per, bar);
      if (!border) bulk_g2s(Pi + p * TB, P.splanes + (size_t)p * nc + i0, per, bar);
    }
    for (int l = 0; l < nl; ++l) {
      bulk_g2s(Nj + l * TB, P.norms + (size_t)l * nc + j0, per, bar);
      if (!border) bulk_g2s(Ni + l * TB, P.norms + (size_t)l * nc + i0, per, bar);
    }
  }
  for (int k = tid; k < sp.nkparams; k += blockDim.x) {
    int type = L_CONSTANT;
    for (int l = 0; l < nl; ++l) {
      const int cnt = sp.leaf[l].type == L_CONSTANT ? 1 : sp.leaf[l].n;
      if (k >= sp.leaf[l].param0 && k < sp.leaf[l].param0 + cnt) type = sp.leaf[l].type;
    }
    ls[k] = transform_param(type, P.theta[k]);
  }
  __syncthreads();
  if (tid < nl) {
    double acc = 0.0;
    const Leaf& L = sp.leaf[tid];
    if (L.type == L_LINEAR)
      for (int k = 0; k < L.n; ++k) acc += 1.0 / ls[L.param0 + k];
    else if (L.type == L_PERIODIC)
      for (int k = 0; k < L.n; ++k) acc += ls[L.param0 + k];
    leaf_c[tid] = acc;
  }
  if (!mbar_wait(bar, 0)) s_fail = 1;
  __syncthreads();
  if (s_fail) {
    if (tid == 0) {
      mbar_wait(bar, 0);  // the copies land (bounded) before the block's shared memory is released
      atomicExch(&P.status[2], 1);
    }
    return;
  }
  const double noise = P.optimise_noise ? P.theta[sp.nkparams] : P.noise;
  const int r0 = (tid & 31) * 2;
  const int c0 = (tid >> 5) * 8;
  double* K = P.K;
  const size_t ld = (size_t)P.ld;
  for (int cc = 0; cc < 8; ++cc) {
    const int c = c0 + cc, j = j0 + c;
    double v[2];
    for (int a = 0; a < 2; ++a) {
      const int r = r0 + a, i = i0 + r;
      double val = 0.0;
      if (border) {
        if (j < P.N && r < P.nrhs)
          val = (r == 0) ? ((P.likelihood == 1) ? P.y[j] : P.y[j] - P.mu[j]) : 1.0;
      } else if (i < P.N && j < P.N) {
        if (i >= j) {
          double stk[MAX_LEAF];
          int top = 0;
          for (int t = 0; t < sp.npost; ++t) {
            const int tok = sp.post[t];
            if (tok >= 0) {
              const Leaf& L = sp.leaf[tok];
              double lv;
              if (L.type == L_RBF) {
                double dot = 0.0;
                for (int k = 0; k < L.n; ++k) dot = fma(Pi[(L.plane0 + k) * TB + r], Pj[(L.plane0 + k) * TB + c], dot);
                const double e = (i == j) ? 0.0 : (Ni[tok * TB + r] + Nj[tok * TB + c]) - 2.0 * dot;
                lv = iexp_neg(-0.5 * e);
              } else if (L.type == L_PERIODIC) {
                double dot = 0.0;
                for (int k = 0; k < 2 * L.n; ++k)
                  dot = fma(Pi[(L.plane0 + k) * TB + r], Pj[(L.plane0 + k) * TB + c], dot);
                lv = (i == j) ? 1.0 : iexp_neg(dot - leaf_c[tok]);
              } else {
                lv = leaf_value(L, Pi, Pj, r, c, ls, sp.cyclic, leaf_c[tok]);
              }
              stk[top++] = lv;
            } else {
              const double b = stk[--top];
              const double a2 = stk[--top];
              stk[top++] = (tok == P_SUM) ? a2 + b : a2 * b;
            }
          }
          val = stk[0];
          if (i == j) val = val + noise * 1.0;
        }
      } else {
        val = (i == j) ? 1.0 : 0.0;
      }
      v[a] = val;
    }
    *reinterpret_cast<double2*>(K + (size_t)j * ld + i0 + r0) = make_double2(v[0], v[1]);
  }
}

// ---------------------------------------------------------------------------
// diagonal block factorisation (blocked, left-looking) + log-det partial
// ---------------------------------------------------------------------------
// W x W block at (col0, col0); W * 4 threads; writes the block's sum of
// log(L_cc) to logdet_part[part].
template <int W>
__global__ void __launch_bounds__(W * 4) k_potf2w(const Prob* __restrict__ probs, int col0_step, int col0_off,
                                                  int part_step, int part_off) {
  const Prob& P = probs[blockIdx.x];
  const int col0 = col0_step + col0_off;
  if (col0 >= P.Nc) return;
  if (*(volatile int*)&P.status[1]) return;
  __shared__ PotfShared<W> sh;
  potf2_block<W>(P, col0, part_step + part_off, threadIdx.x, sh, 0);
}

// ---------------------------------------------------------------------------
// panel solve: A21 <- A21 * L11^-T for the rows below the W x W diagonal
// block at col0, in tiles of 64 rows (including the border rows of
// right-hand sides; rows past the last 64-row tile of the problem are skipped)
// ---------------------------------------------------------------------------
template <int W>
__global__ void __launch_bounds__(256) k_trsmw(const Prob* __restrict__ probs, int col0_step, int col0_off) {
  const Prob& P = probs[blockIdx.y];
  const int col0 = col0_step + col0_off;
  const int last = P.nrt ? P.nrt - 1 : P.nsteps;  // last 64-row tile
  const int row_end = (last + 1) * TB;
  const int r0 = col0 + W + blockIdx.x * TB;
  if (col0 >= P.Nc || r0 >= row_end) return;
  if (*(volatile int*)&P.status[1]) return;
  // the adjoint's identity rows: zero panel values before their own panel
  // (see k_update), so their solve at earlier panels would leave zeros
  if (r0 / TB > P.nsteps && r0 / TB - (P.nsteps + 1) > col0 / TB) return;
  if (P.border_only && r0 / TB <= P.nsteps) return;  // the factor is final: identity rows only
  constexpr int LDA = TB + 1;
  __shared__ double L[W * (W + 1)];
  __shared__ double B[W * LDA];
  __shared__ double rd[W];
  const int tid = threadIdx.x;
  const size_t ld = (size_t)P.ld;
  const int nr = min(TB, row_end - r0);
  const double* Ld = P.K + (size_t)col0 * ld + col0;
  double* Bd = P.K + (size_t)col0 * ld + r0;
  for (int e = tid; e < W * W; e += blockDim.x) {
    const int r = e % W, c = e / W;
    L[c * (W + 1) + r] = Ld[(size_t)c * ld + r];
  }
  for (int e = tid; e < TB * W; e += blockDim.x) {
    const int r = e % TB, c = e / TB;
    B[c * LDA + r] = r < nr ? Bd[(size_t)c * ld + r] : 0.0;
  }
  __syncthreads();
  if (tid < W) rd[tid] = 1.0 / L[tid * (W + 1) + tid];
  __syncthreads();
  for (int c = 0; c < W; ++c) {
    if (tid < TB) B[c * LDA + tid] *= rd[c];
    __syncthreads();
    const int w = W - 1 - c;
    for (int e = tid; e < w * TB; e += blockDim.x) {
      const int r = e % TB, q = c + 1 + e / TB;
      B[q * LDA + r] = fma(-B[c * LDA + r], L[c * (W + 1) + q], B[q * LDA + r]);
    }
    __syncthreads();
  }
  for (int e = tid; e < TB * W; e += blockDim.x) {
    const int r = e % TB, c = e / TB;
    if (r < nr) Bd[(size_t)c * ld + r] = B[c * LDA + r];
  }
}

// ---------------------------------------------------------------------------
// trailing update C(ti, tj) -= P(ti) P(tj)^T on the FP64 MMA pipe
// (mma.sync m8n8k4 f64).  128 threads, 4 warps x (32 x 32).
// ---------------------------------------------------------------------------
constexpr int UPD_STRIDE = TB + 8;  // k-major staging, 8-double pad

__device__ __forceinline__ void dmma_8x8x4(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

__global__ void __launch_bounds__(128) k_update(const Prob* __restrict__ probs, int step) {
  const Prob& P = probs[blockIdx.z];
  const int ti = step + 1 + blockIdx.x, tj = step + 1 + blockIdx.y;
  const int last = P.nrt ? P.nrt - 1 : P.nsteps;
  if (step >= P.nsteps || tj >= P.nsteps || ti > last || ti < tj) return;
  // The adjoint's identity rows (row tiles after the right-hand-side tile):
  // tile nsteps + 1 + q starts as the unit rows of tile q, whose panel values
  // stay exactly zero before panel q (L^-1 is lower triangular), so there
  // is nothing to subtract at earlier steps.
  if (ti > P.nsteps && ti - (P.nsteps + 1) > step) return;
  if (P.border_only && ti <= P.nsteps) return;  // the factor is final: identity rows only
  if (*(volatile int*)&P.status[1]) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* As = reinterpret_cast<double*>(smem_raw);  // [k][m]
  double* Bs = As + TB * UPD_STRIDE;                  // [k][n]
  const int tid = threadIdx.x;
  const size_t ld = (size_t)P.ld;
  const double* Ag = P.K + (size_t)(step * TB) * ld + ti * TB;
  const double* Bg = P.K + (size_t)(step * TB) * ld + tj * TB;
  // 64 columns x 64 rows each; a warp moves one column (32 x double2) per pass
  for (int e = tid; e < TB * (TB / 2); e += blockDim.x) {
    const int k = e / (TB / 2), m2 = (e % (TB / 2)) * 2;
    const double2 a = *reinterpret_cast<const double2*>(Ag + (size_t)k * ld + m2);
    const double2 b = *reinterpret_cast<const double2*>(Bg + (size_t)k * ld + m2);
    *reinterpret_cast<double2*>(As + k * UPD_STRIDE + m2) = a;
    *reinterpret_cast<double2*>(Bs + k * UPD_STRIDE + m2) = b;
  }
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  double acc[4][4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;
  const int lr = lane >> 2, lk = lane & 3;
#pragma unroll 2
  for (int k0 = 0; k0 < TB; k0 += 4) {
    double af[4], bf[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) af[a] = As[(k0 + lk) * UPD_STRIDE + wm + a * 8 + lr];
#pragma unroll
    for (int b = 0; b < 4; ++b) bf[b] = Bs[(k0 + lk) * UPD_STRIDE + wn + b * 8 + lr];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) dmma_8x8x4(acc[a][b][0], acc[a][b][1], af[a], bf[b]);
  }
  double* Cg = P.K + (size_t)(tj * TB) * ld + ti * TB;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int m = wm + a * 8 + lr;
      const int n = wn + b * 8 + lk * 2;
      double* c0p = Cg + (size_t)n * ld + m;
      double* c1p = Cg + (size_t)(n + 1) * ld + m;
      *c0p = *c0p - acc[a][b][0];
      *c1p = *c1p - acc[a][b][1];
    }
}

// ---------------------------------------------------------------------------
// likelihood epilogue (likelihood.f90:161-253) from the border rows
// ---------------------------------------------------------------------------
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  if (threadIdx.x == 0) red[0] = s;
  __syncthreads();
  return red[0];
}

__global__ void __launch_bounds__(256) k_finalize(const Prob* __restrict__ probs) {
  const Prob& P = probs[blockIdx.x];
  __shared__ double red[32];
  const int tid = threadIdx.x;
  const int N = P.N;
  if (P.status[1] || P.status[2] || P.status[3]) {
    if (tid == 0) {
      // -1: a bounded wait gave up; -2: a panel value broke its row's scale bound
      const int info = P.status[2] ? -1 : (P.status[3] && !P.status[1] ? -2 : P.status[0]);
      P.out[0] = nan("");
      P.status[0] = info;
      if (P.ll_dst) *P.ll_dst = nan("");
      if (P.info_dst) *P.info_dst = info;
    }
    return;
  }
  const size_t ld = (size_t)P.ld;
  const double* z0 = P.K + P.Nc;      // row Nc: r_0 = y - mu (marginal) or y (concentrated)
  const double* z1 = P.K + P.Nc + 1;  // row Nc+1: ones (concentrated)
  double logdet = 0.0;
  if (tid == 0) {
    const int nparts = P.mode == 1 ? P.Nc / QW : P.nsteps;  // 32-column parts in tensor-core mode
    for (int s = 0; s < nparts; ++s) logdet += P.logdet_part[s];
    logdet *= 2.0;
  }
  double ll, mean = 0.0, s2 = 0.0;
  if (P.likelihood == 0) {
    double q = 0.0;
    for (int j = tid; j < N; j += blockDim.x) {
      const double v = z0[(size_t)j * ld];
      q = fma(v, v, q);
      P.z[j] = v;
    }
    q = block_sum(q, red);
    ll = -0.5 * q - 0.5 * logdet - 0.5 * (double)N * FGPU_LOG_TWOPI;
  } else {
    double a = 0.0, b = 0.0;
    for (int j = tid; j < N; j += blockDim.x) {
      const double u = z0[(size_t)j * ld], v = z1[(size_t)j * ld];
      a = fma(v, u, a);
      b = fma(v, v, b);
    }
    a = block_sum(a, red);
    b = block_sum(b, red);
    mean = a / b;  // 1^T K^-1 y / 1^T K^-1 1 (likelihood.f90:229)
    double q = 0.0;
    for (int j = tid; j < N; j += blockDim.x) {
      const double w = z0[(size_t)j * ld] - mean * z1[(size_t)j * ld];
      q = fma(w, w, q);
      P.z[j] = w;
    }
    q = block_sum(q, red);
    s2 = q / (double)N;  // (y - mu)^T K^-1 (y - mu) / N (likelihood.f90:239)
    ll = -0.5 * (double)N * log(s2) - 0.5 * logdet;
  }
  for (int j = N + tid; j < P.Nc; j += blockDim.x) P.z[j] = 0.0;
  if (tid == 0) {
    P.out[0] = ll;
    P.out[1] = logdet;
    P.out[2] = mean;
    P.out[3] = s2;
    P.status[0] = 0;
    if (P.ll_dst) *P.ll_dst = ll;
    if (P.info_dst) *P.info_dst = 0;
  }
}

// ---------------------------------------------------------------------------
// alpha = L^-T z by blocked back-substitution (dpotrs's second half)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TB) k_bs_diag(const Prob* __restrict__ probs, int blk) {
  const Prob& P = probs[blockIdx.x];
  if (blk >= P.nsteps || P.status[1] || P.status[2]) return;
  __shared__ double L[TB * (TB + 1)];
  __shared__ double z[TB];
  const int tid = threadIdx.x;
  const size_t ld = (size_t)P.ld;
  const double* Ld = P.K + (size_t)(blk * TB) * ld + blk * TB;
  for (int c = 0; c < TB; ++c) L[c * (TB + 1) + tid] = Ld[(size_t)c * ld + tid];
  z[tid] = P.z[blk * TB + tid];
  __syncthreads();
  for (int c = TB - 1; c >= 0; --c) {
    if (tid == 0) z[c] = z[c] / L[c * (TB + 1) + c];
    __syncthreads();
    if (tid < c) z[tid] = fma(-L[tid * (TB + 1) + c], z[c], z[tid]);
    __syncthreads();
  }
  P.z[blk * TB + tid] = z[tid];
}

// z[0 : blk*TB) -= L[blk rows, 0 : blk*TB)^T alpha_blk; one warp per column.
__global__ void __launch_bounds__(256) k_bs_update(const Prob* __restrict__ probs, int blk) {
  const Prob& P = probs[blockIdx.y];
  if (blk >= P.nsteps || P.status[1] || P.status[2]) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int col = blockIdx.x * 8 + warp;
  if (col >= blk * TB) return;
  const size_t ld = (size_t)P.ld;
  const double* Lc = P.K + (size_t)col * ld + blk * TB;
  const double* ab = P.z + blk * TB;
  double s = fma(Lc[lane], ab[lane], Lc[lane + 32] * ab[lane + 32]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) P.z[col] -= s;
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
static std::atomic<unsigned> g_smem_done[64];

cudaError_t ensure_smem_attr(const void* func, int slot, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned bit = 1u << slot;
  if (dev >= 0 && dev < 64 && (g_smem_done[dev].load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64) g_smem_done[dev].fetch_or(bit, std::memory_order_release);
  return cudaSuccess;
}

cudaError_t launch_build(const Prob* probs, int nprob, int max_nsteps, int max_nplanes, cudaStream_t s) {
  const size_t smem = build_smem_bytes(max_nplanes);
  cudaError_t e = ensure_smem_attr((const void*)k_build, SMEM_BUILD, (int)build_smem_bytes(MAX_PLANES));
  if (e != cudaSuccess) return e;
  dim3 grid(max_nsteps + 1, max_nsteps, nprob);
  k_build<<<grid, 256, smem, s>>>(probs);
  return cudaGetLastError();
}

cudaError_t launch_prep_planes(const Prob* probs, int nprob, int max_nc, cudaStream_t s) {
  k_prep_planes<<<dim3((max_nc + 255) / 256, MAX_LEAF, nprob), 256, 0, s>>>(probs);
  return cudaGetLastError();
}

cudaError_t launch_build_dot(const Prob* probs, int nprob, int max_nsteps, int max_nplanes, cudaStream_t s) {
  cudaError_t e = ensure_smem_attr((const void*)k_build_dot, SMEM_BUILD_DOT, (int)build_dot_smem_bytes(MAX_PLANES));
  if (e != cudaSuccess) return e;
  dim3 grid(max_nsteps + 1, max_nsteps, nprob);
  k_build_dot<<<grid, 256, build_dot_smem_bytes(max_nplanes), s>>>(probs);
  return cudaGetLastError();
}

cudaError_t launch_potf2(const Prob* probs, int nprob, int step, cudaStream_t s) {
  k_potf2w<TB><<<nprob, TB * 4, 0, s>>>(probs, step * TB, 0, step, 0);
  return cudaGetLastError();
}

cudaError_t launch_potf2_quarter(const Prob* probs, int nprob, int step, int q, cudaStream_t s) {
  // log-det parts indexed by 32-column block
  k_potf2w<QW><<<nprob, QW * 4, 0, s>>>(probs, step * NB, q * QW, step * (NB / QW), q);
  return cudaGetLastError();
}

cudaError_t launch_trsm(const Prob* probs, int nprob, int step, int max_nsteps, cudaStream_t s,
                        int max_rowtiles) {
  if (max_rowtiles <= 0) max_rowtiles = max_nsteps + 1;
  const int rows = max_rowtiles - step - 1;  // row tiles step+1 .. last (incl. border rows)
  if (rows <= 0) return cudaSuccess;
  k_trsmw<TB><<<dim3(rows, nprob), 256, 0, s>>>(probs, step * TB, 0);
  return cudaGetLastError();
}

cudaError_t launch_update(const Prob* probs, int nprob, int step, int max_nsteps, cudaStream_t s,
                          int max_rowtiles) {
  if (max_rowtiles <= 0) max_rowtiles = max_nsteps + 1;
  const int m = max_nsteps - step - 1;  // trailing column tiles
  const int mr = max_rowtiles - step - 1;  // trailing row tiles incl. border rows
  if (m <= 0) return cudaSuccess;
  const int smem = 2 * TB * UPD_STRIDE * (int)sizeof(double);
  cudaError_t e = ensure_smem_attr((const void*)k_update, SMEM_UPDATE, smem);
  if (e != cudaSuccess) return e;
  k_update<<<dim3(mr, m, nprob), 128, smem, s>>>(probs, step);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const Prob* probs, int nprob, cudaStream_t s) {
  k_finalize<<<nprob, 256, 0, s>>>(probs);
  return cudaGetLastError();
}

cudaError_t launch_backsolve(const Prob* probs, int nprob, int max_nsteps, double* /*alpha_out*/,
                             cudaStream_t s, long long* nlaunch) {
  for (int b = max_nsteps - 1; b >= 0; --b) {
    k_bs_diag<<<nprob, TB, 0, s>>>(probs, b);
    if (nlaunch) ++*nlaunch;
    if (b > 0) {
      k_bs_update<<<dim3((b * TB + 7) / 8, nprob), 256, 0, s>>>(probs, b);
      if (nlaunch) ++*nlaunch;
    }
  }
  return cudaGetLastError();
}

}  // namespace fgpu

// ---------------------------------------------------------------------------
// diagnostic: the device exponential of the kernel-matrix builds on host values
// ---------------------------------------------------------------------------
namespace fgpu {
__global__ void k_diag_exp(const double* __restrict__ x, double* __restrict__ y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = iexp_neg(x[i]);
}
}  // namespace fgpu

extern "C" int fgpu_diag_exp(const double* x, double* y, int n) {
  using namespace fgpu;
  internal_clear_error();
  if (n < 0 || (n > 0 && (!x || !y))) return internal_fail(FGPU_EINVAL, "fgpu_diag_exp: bad arguments");
  if (n == 0) return FGPU_OK;
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * 2 * (size_t)n);
  if (e != cudaSuccess) return internal_fail(FGPU_ENOMEM, cudaGetErrorString(e));
  if ((e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice)) == cudaSuccess) {
    k_diag_exp<<<(n + 255) / 256, 256>>>(d, d + n, n);
    internal_add_launches(1);
    if ((e = cudaGetLastError()) == cudaSuccess)
      e = cudaMemcpy(y, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  if (e != cudaSuccess) return internal_fail(FGPU_ECUDA, cudaGetErrorString(e));
  return FGPU_OK;
}

// ---------------------------------------------------------------------------
// diagnostic: the kernels' bounded mbarrier wait giving up.  One warp waits
// on a shared-memory mbarrier that nothing arrives on (arrive = 0) or that
// its lane 0 has completed first (arrive = 1), with `polls` polls, through
// the same helper the tensor-core kernels use, and records a give-up in
// status[2] as they do.  Nothing asynchronous (copy, MMA) is issued, so
// nothing is left in flight when the wait gives up.
// ---------------------------------------------------------------------------
namespace fgpu {
__global__ void k_diag_wait(int* __restrict__ status, int polls, int arrive) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (threadIdx.x == 0 && arrive) mbar_arrive(&bar);
  __syncwarp();
  const bool ok = mbar_wait_n(&bar, 0, polls);
  if (threadIdx.x == 0 && !ok) atomicExch(&status[2], 1);
}
}  // namespace fgpu

extern "C" int fgpu_diag_wait(int polls, int arrive) {
  using namespace fgpu;
  internal_clear_error();
  if (polls < 1 || polls > (1 << 22) || (arrive != 0 && arrive != 1))
    return internal_fail(FGPU_EINVAL, "fgpu_diag_wait: polls must be in 1..2^22 and arrive 0 or 1");
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int) * 4);
  if (e != cudaSuccess) return internal_fail(FGPU_ENOMEM, cudaGetErrorString(e));
  int h[4] = {0, 0, 0, 0};
  if ((e = cudaMemset(d, 0, sizeof(int) * 4)) == cudaSuccess) {
    k_diag_wait<<<1, 32>>>(d, polls, arrive);
    internal_add_launches(1);
    if ((e = cudaGetLastError()) == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  if (e != cudaSuccess) return internal_fail(FGPU_ECUDA, cudaGetErrorString(e));
  // the status word maps to the host error exactly as after an evaluation
  if (h[2]) return internal_fail(FGPU_ETIMEOUT, "a bounded wait in a kernel gave up (copy or MMA)");
  return FGPU_OK;
}

// ---------------------------------------------------------------------------
// diagnostic: the kernel-matrix build's leaf-scale exponential,
// y[i] = exp(-E[i] 2^e), on host values
// ---------------------------------------------------------------------------
namespace fgpu {
__global__ void k_diag_exp_fixed(const unsigned long long* __restrict__ E, int e, double* __restrict__ y, int n) {
  __shared__ unsigned long long tab[1024], fine[1024];
  for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
    tab[k] = g_iexp_tab1024[k];
    fine[k] = g_iexp_fine1024[k];
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = iexp_fixed_tab(E[i], iexp_scale(e), tab, fine);
}
}  // namespace fgpu

extern "C" int fgpu_diag_exp_fixed(const unsigned long long* E, int e, double* y, int n) {
  using namespace fgpu;
  internal_clear_error();
  if (n < 0 || (n > 0 && (!E || !y)) || e > -1 || e < -128)
    return internal_fail(FGPU_EINVAL, "fgpu_diag_exp_fixed: bad arguments (e must be in -128..-1)");
  if (n == 0) return FGPU_OK;
  unsigned long long* d = nullptr;
  cudaError_t err = cudaMalloc(&d, sizeof(unsigned long long) * 2 * (size_t)n);
  if (err != cudaSuccess) return internal_fail(FGPU_ENOMEM, cudaGetErrorString(err));
  double* yd = reinterpret_cast<double*>(d + n);
  if ((err = cudaMemcpy(d, E, sizeof(unsigned long long) * n, cudaMemcpyHostToDevice)) == cudaSuccess) {
    k_diag_exp_fixed<<<(n + 255) / 256, 256>>>(d, e, yd, n);
    internal_add_launches(1);
    if ((err = cudaGetLastError()) == cudaSuccess)
      err = cudaMemcpy(y, yd, sizeof(double) * n, cudaMemcpyDeviceToHost);
  }
  cudaFree(d);
  if (err != cudaSuccess) return internal_fail(FGPU_ECUDA, cudaGetErrorString(err));
  return FGPU_OK;
}
