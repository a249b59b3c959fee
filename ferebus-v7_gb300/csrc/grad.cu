// Adjoint of the log-likelihood (FP64):
//   d logL / d theta_q = 1/2 sum_ij W_ij dK_ij/dtheta_q,  W = alpha alpha^T / s - K^-1,
// s = 1 (marginal) or sigma^2 (concentrated; the profiled mean and variance
// drop out by the envelope theorem), and dK/dnoise = I.
//
// K^-1: the factorisation runs on a taller matrix whose rows below the
// right-hand-side tile start as the identity; the sweep turns them into
// B = L^-T (row i of B = column i of L^-1, zero left of column i), and
// K^-1 = B B^T.  dK/dtheta is never stored: the fused pass recomputes the
// leaf values and their per-feature factors from the feature planes tile by
// tile, exactly as the kernel-matrix build does.
#include "fgpu_internal.h"
#include "iexp.cuh"

#include <cmath>

namespace fgpu {

namespace {
constexpr int GCHUNK = 32;  // parameters per pass of the fused kernel (+ 1 noise slot)
constexpr int USTRIDE = TB + 8;
__device__ __forceinline__ void dmma(double& c0, double& c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}
}  // namespace

// rows Nc + 64 + q: e_q^T for q < N, zero otherwise
__global__ void __launch_bounds__(256) k_identity_border(const Prob* __restrict__ pp) {
  const Prob& P = *pp;
  const int ct = blockIdx.x, rt = blockIdx.y;
  const size_t ld = (size_t)P.ld;
  const int r0 = P.Nc + TB + rt * TB;
  for (int e = threadIdx.x; e < TB * TB; e += blockDim.x) {
    const int r = e % TB, c = e / TB;
    const int q = rt * TB + r, j = ct * TB + c;
    P.K[(size_t)j * ld + r0 + r] = (q == j && q < P.N) ? 1.0 : 0.0;
  }
}

// K^-1 tile (ti, tj), ti >= tj: sum over k-blocks kb >= ti of B[ti, kb] B[tj, kb]^T
__global__ void __launch_bounds__(128) k_syrk_inv(const Prob* __restrict__ pp) {
  const Prob& P = *pp;
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (ti < tj || ti >= P.nsteps) return;
  extern __shared__ __align__(16) double smg[];
  double* As = smg;                 // [k][m]
  double* Bs = smg + TB * USTRIDE;  // [k][n]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const size_t ld = (size_t)P.ld;
  const int R0 = P.Nc + TB;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32, lr = lane >> 2, lk = lane & 3;
  double acc[4][4][2];
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;
  for (int kb = ti; kb < P.nsteps; ++kb) {
    const double* Ag = P.K + (size_t)(kb * TB) * ld + R0 + ti * TB;
    const double* Bg = P.K + (size_t)(kb * TB) * ld + R0 + tj * TB;
    __syncthreads();
    for (int e = tid; e < TB * (TB / 2); e += blockDim.x) {
      const int k = e / (TB / 2), m2 = (e % (TB / 2)) * 2;
      *reinterpret_cast<double2*>(As + k * USTRIDE + m2) = *reinterpret_cast<const double2*>(Ag + (size_t)k * ld + m2);
      *reinterpret_cast<double2*>(Bs + k * USTRIDE + m2) = *reinterpret_cast<const double2*>(Bg + (size_t)k * ld + m2);
    }
    __syncthreads();
    for (int k0 = 0; k0 < TB; k0 += 4) {
      double af[4], bf[4];
      for (int a = 0; a < 4; ++a) af[a] = As[(k0 + lk) * USTRIDE + wm + a * 8 + lr];
      for (int b = 0; b < 4; ++b) bf[b] = Bs[(k0 + lk) * USTRIDE + wn + b * 8 + lr];
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) dmma(acc[a][b][0], acc[a][b][1], af[a], bf[b]);
    }
  }
  const size_t nc = (size_t)P.Nc;
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      const int m = ti * TB + wm + a * 8 + lr;
      const int n = tj * TB + wn + b * 8 + lk * 2;
      P.kinv[(size_t)n * nc + m] = acc[a][b][0];
      P.kinv[(size_t)(n + 1) * nc + m] = acc[a][b][1];
    }
}

// Fused dK/dtheta pass over the lower tiles; partial sums per CTA for the
// parameters [q0, q0 + GCHUNK) and (slot GCHUNK) the noise.
__global__ void __launch_bounds__(256) k_grad(const Prob* __restrict__ pp, int q0) {
  const Prob& P = *pp;
  const int ti = blockIdx.x, tj = blockIdx.y;
  const int cta = blockIdx.y * gridDim.x + blockIdx.x;
  __shared__ double ls[MAX_PARAMS];
  __shared__ double red[8][GCHUNK + 1];
  __shared__ int lchild[MAX_POST], rchild[MAX_POST];
  const Spec& sp = *P.spec;
  const int tid = threadIdx.x;
  double acc[GCHUNK + 1];
  for (int q = 0; q <= GCHUNK; ++q) acc[q] = 0.0;
  const bool work = ti >= tj && ti < P.nsteps && !P.status[1];
  if (tid == 0) {
    int stk[MAX_POST], top = 0;
    for (int t = 0; t < sp.npost; ++t) {
      lchild[t] = rchild[t] = -1;
      if (sp.post[t] < 0) {
        rchild[t] = stk[--top];
        lchild[t] = stk[--top];
      }
      stk[top++] = t;
    }
  }
  for (int k = tid; k < sp.nkparams; k += blockDim.x) {
    int type = L_CONSTANT;
    for (int l = 0; l < sp.nleaf; ++l) {
      const int cnt = sp.leaf[l].type == L_CONSTANT ? 1 : sp.leaf[l].n;
      if (k >= sp.leaf[l].param0 && k < sp.leaf[l].param0 + cnt) type = sp.leaf[l].type;
    }
    const double t = P.theta[k];
    ls[k] = (type == L_RBF || type == L_RBF_CYCLIC) ? exp(t)
            : (type == L_PERIODIC) ? (1.0 / exp(t)) * (1.0 / exp(t))
            : (type == L_LINEAR) ? exp(-t) : t;
  }
  __syncthreads();
  if (work) {
    const double s2 = P.likelihood == 1 ? P.out[3] : 1.0;
    const size_t nc = (size_t)P.Nc;
    const double* X = P.planes;
    const int r0 = (tid & 31) * 2, c0 = (tid >> 5) * 8;
    for (int cc = 0; cc < 8; ++cc)
      for (int a = 0; a < 2; ++a) {
        const int i = ti * TB + r0 + a, j = tj * TB + c0 + cc;
        if (i < j || i >= P.N || j >= P.N) continue;
        const double w = (P.z[i] * P.z[j] / s2 - P.kinv[(size_t)j * nc + i]) * (i == j ? 1.0 : 2.0);
        if (i == j) acc[GCHUNK] += w;
        // forward: leaf values
        double val[MAX_POST], adj[MAX_POST];
        for (int t = 0; t < sp.npost; ++t) {
          const int tok = sp.post[t];
          adj[t] = 0.0;
          if (tok >= 0) {
            const Leaf& L = sp.leaf[tok];
            double e = 0.0, v;
            if (L.type == L_RBF || L.type == L_RBF_CYCLIC) {
              for (int k = 0; k < L.n; ++k) {
                double d = X[(size_t)(L.plane0 + k) * nc + i] - X[(size_t)(L.plane0 + k) * nc + j];
                if (L.type == L_RBF_CYCLIC && sp.cyclic[L.plane0 + k]) {
                  const double aa = fabs(d) + 3.141592653589793;
                  d = copysign(1.0, d) * (fmod(aa, 6.283185307179586) - 3.141592653589793);
                }
                e = fma(ls[L.param0 + k], d * d, e);
              }
              v = iexp_neg(-0.5 * e);
            } else if (L.type == L_PERIODIC) {
              for (int k = 0; k < L.n; ++k) {
                const double si = X[(size_t)(L.plane0 + 2 * k) * nc + i], ci = X[(size_t)(L.plane0 + 2 * k + 1) * nc + i];
                const double sj = X[(size_t)(L.plane0 + 2 * k) * nc + j], cj = X[(size_t)(L.plane0 + 2 * k + 1) * nc + j];
                const double tt = fma(si, cj, -(ci * sj));
                e = fma(ls[L.param0 + k], tt * tt, e);
              }
              v = iexp_neg(-2.0 * e);
            } else if (L.type == L_LINEAR) {
              v = 0.0;
              for (int k = 0; k < L.n; ++k) v += 1.0 / ls[L.param0 + k];
            } else {
              v = ls[L.param0];
            }
            val[t] = v;
          } else {
            val[t] = (tok == P_SUM) ? val[lchild[t]] + val[rchild[t]] : val[lchild[t]] * val[rchild[t]];
          }
        }
        // backward: sensitivity of K to every node
        adj[sp.npost - 1] = 1.0;
        for (int t = sp.npost - 1; t >= 0; --t) {
          const int tok = sp.post[t];
          if (tok < 0) {
            const int l = lchild[t], r = rchild[t];
            if (tok == P_SUM) {
              adj[l] += adj[t];
              adj[r] += adj[t];
            } else {
              adj[l] += adj[t] * val[r];
              adj[r] += adj[t] * val[l];
            }
          }
        }
        // per-parameter factors
        for (int t = 0; t < sp.npost; ++t) {
          const int tok = sp.post[t];
          if (tok < 0) continue;
          const Leaf& L = sp.leaf[tok];
          const double cw = w * adj[t];
          const int cnt = L.type == L_CONSTANT ? 1 : L.n;
          if (L.param0 + cnt <= q0 || L.param0 >= q0 + GCHUNK) continue;
          for (int k = 0; k < cnt; ++k) {
            const int q = L.param0 + k - q0;
            if (q < 0 || q >= GCHUNK) continue;
            double dv;
            if (L.type == L_RBF || L.type == L_RBF_CYCLIC) {
              double d = X[(size_t)(L.plane0 + k) * nc + i] - X[(size_t)(L.plane0 + k) * nc + j];
              if (L.type == L_RBF_CYCLIC && sp.cyclic[L.plane0 + k]) {
                const double aa = fabs(d) + 3.141592653589793;
                d = copysign(1.0, d) * (fmod(aa, 6.283185307179586) - 3.141592653589793);
              }
              dv = val[t] * (-0.5 * ls[L.param0 + k] * d * d);
            } else if (L.type == L_PERIODIC) {
              const double si = X[(size_t)(L.plane0 + 2 * k) * nc + i], ci = X[(size_t)(L.plane0 + 2 * k + 1) * nc + i];
              const double sj = X[(size_t)(L.plane0 + 2 * k) * nc + j], cj = X[(size_t)(L.plane0 + 2 * k + 1) * nc + j];
              const double tt = fma(si, cj, -(ci * sj));
              dv = val[t] * (4.0 * ls[L.param0 + k] * tt * tt);
            } else if (L.type == L_LINEAR) {
              dv = 1.0 / ls[L.param0 + k];  // d exp(theta) / d theta
            } else {
              dv = 1.0;
            }
            acc[q] += cw * dv;
          }
        }
      }
  }
  // block reduction in a fixed order
  const int warp = tid >> 5, lane = tid & 31;
  for (int q = 0; q <= GCHUNK; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (tid <= GCHUNK) {
    double v = 0.0;
    for (int w = 0; w < 8; ++w) v += red[w][tid];
    P.gpart[(size_t)cta * (GCHUNK + 1) + tid] = v;
  }
}

__global__ void k_grad_reduce(const Prob* __restrict__ pp, int nblocks, int q0, int nk, int noise_slot,
                              double* __restrict__ g) {
  const Prob& P = *pp;
  const int q = threadIdx.x;
  if (q > GCHUNK) return;
  double v = 0.0;
  for (int b = 0; b < nblocks; ++b) v += P.gpart[(size_t)b * (GCHUNK + 1) + q];
  if (q < GCHUNK && q0 + q < nk) g[q0 + q] = 0.5 * v;
  if (q == GCHUNK && noise_slot >= 0) g[noise_slot] = 0.5 * v;
}

cudaError_t launch_identity_border(const Prob* p, int nc, cudaStream_t s) {
  k_identity_border<<<dim3(nc / TB, nc / TB), 256, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_syrk_inv(const Prob* p, int nsteps, cudaStream_t s) {
  const int smem = 2 * TB * USTRIDE * (int)sizeof(double);
  cudaError_t e = ensure_smem_attr((const void*)k_syrk_inv, SMEM_SYRK, smem);
  if (e != cudaSuccess) return e;
  k_syrk_inv<<<dim3(nsteps, nsteps), 128, smem, s>>>(p);
  return cudaGetLastError();
}

// Driver used by the host: all chunks, kernel passes and reductions.
cudaError_t enqueue_grad_passes(const Prob* p, int nsteps, int nk, int optimise_noise, double* g_out,
                                cudaStream_t s, long long* nlaunch) {
  const int nblocks = nsteps * nsteps;
  for (int q0 = 0; q0 < (nk > 0 ? nk : 1); q0 += GCHUNK) {
    k_grad<<<dim3(nsteps, nsteps), 256, 0, s>>>(p, q0);
    k_grad_reduce<<<1, GCHUNK + 1, 0, s>>>(p, nblocks, q0, nk, (q0 == 0 && optimise_noise) ? nk : -1, g_out);
    if (nlaunch) *nlaunch += 2;
  }
  return cudaGetLastError();
}

}  // namespace fgpu
