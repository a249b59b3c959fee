// The W x W diagonal-block Cholesky (FP64) with its log-det part, as a
// block-level device routine for W * 4 threads synchronised by one hardware
// barrier: called by its own kernel (barrier 0 = the whole CTA) and by the
// tensor-core coupling kernel, whose four epilogue warps factor the next
// quarter's diagonal block as soon as they have coupled into it (barrier 1).
//
// Blocked left-looking factorisation in shared memory, panels of 8 columns
// (the dot-product order of LAPACK's dpotf2, lapack/dpotf2.f): (a) the panel
// minus the finished columns times their rows, all threads; (b) the 8 x 8
// diagonal block by one warp in registers (shuffles, no block barrier);
// (c) the rows below by forward substitution, one thread per row.  Three
// barriers per panel.  A non-positive pivot sets the problem's LAPACK-style
// info (1-based column) and failed flag.
#pragma once
#include "fgpu_internal.h"

namespace fgpu {

template <int W>
struct PotfShared {
  double A[W * (W + 1)];  // A[c * (W + 1) + r]
  double rdg[W];          // 1 / L_cc
  int fail_col;
};

__device__ __forceinline__ void bar_sync_n(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <int W>
__device__ __forceinline__ void potf2_block(const Prob& P, int col0, int part, int tid, PotfShared<W>& sh, int bar) {
  constexpr int LDA = W + 1;
  constexpr int NT = W * 4;
  double* A = sh.A;
  const int lane = tid & 31, warp = tid >> 5;
  const size_t ld = (size_t)P.ld;
  double* Kd = P.K + (size_t)col0 * ld + col0;
  for (int e = tid; e < W * W; e += NT) {
    const int r = e % W, c = e / W;
    A[c * LDA + r] = Kd[(size_t)c * ld + r];
  }
  if (tid == 0) sh.fail_col = -1;
  bar_sync_n(bar, NT);
  for (int c0 = 0; c0 < W; c0 += 8) {
    // (a) columns c0..c0+7, rows >= column: subtract sum_{k < c0} L_rk L_ck
    if (c0 > 0) {
      const int r = tid % W, cp = c0 + 2 * (tid / W);
      if (r >= cp) {
        double a0 = A[cp * LDA + r], a1 = A[(cp + 1) * LDA + r];
        for (int k = 0; k < c0; ++k) {
          const double l = A[k * LDA + r];
          a0 = fma(-l, A[k * LDA + cp], a0);
          a1 = fma(-l, A[k * LDA + cp + 1], a1);
        }
        A[cp * LDA + r] = a0;
        if (r > cp) A[(cp + 1) * LDA + r] = a1;
      }
    }
    bar_sync_n(bar, NT);
    // (b) 8 x 8 diagonal block: lane i < 8 holds row c0 + i
    if (warp == 0) {
      double v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = (lane < 8 && k <= lane) ? A[(c0 + k) * LDA + c0 + lane] : 0.0;
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const double d = __shfl_sync(0xffffffffu, v[jj], jj);
        if (!(d > 0.0)) {  // d is the same in every lane: the warp leaves together
          if (lane == 0) sh.fail_col = c0 + jj;
          break;
        }
        const double sd = sqrt(d);
        const double rd = 1.0 / sd;
        if (lane == jj) v[jj] = sd;
        if (lane > jj) v[jj] *= rd;
#pragma unroll
        for (int c = jj + 1; c < 8; ++c) {
          const double lcj = __shfl_sync(0xffffffffu, v[jj], c);
          if (lane >= c) v[c] = fma(-v[jj], lcj, v[c]);
        }
        if (lane == 0) sh.rdg[c0 + jj] = rd;
      }
      if (lane < 8) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k <= lane) A[(c0 + k) * LDA + c0 + lane] = v[k];
      }
    }
    bar_sync_n(bar, NT);
    if (sh.fail_col >= 0) break;
    // (c) rows below the diagonal block: forward substitution over the panel
    if (tid < W - c0 - 8) {
      const int r = c0 + 8 + tid;
      double x[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        double a = A[(c0 + c) * LDA + r];
#pragma unroll
        for (int k = 0; k < c; ++k) a = fma(-x[k], A[(c0 + k) * LDA + c0 + c], a);
        x[c] = a * sh.rdg[c0 + c];
        A[(c0 + c) * LDA + r] = x[c];
      }
    }
    bar_sync_n(bar, NT);
  }
  if (sh.fail_col >= 0) {
    if (tid == 0) {
      P.status[0] = col0 + sh.fail_col + 1;  // LAPACK info: 1-based column
      P.status[1] = 1;
    }
    return;
  }
  for (int e = tid; e < W * W; e += NT) {
    const int r = e % W, c = e / W;
    if (r >= c) Kd[(size_t)c * ld + r] = A[c * LDA + r];
  }
  // log-det partial: 2 * sum log(L_jj) is formed in the epilogue
  // (arith.f90:72-93); here the block's sum of logs, in column order.
  if (tid < 32) {
    double sl = 0.0;
    for (int c = tid * (W / 32); c < (tid + 1) * (W / 32); ++c) sl += log(A[c * LDA + c]);
    for (int o = 16; o > 0; o >>= 1) sl += __shfl_down_sync(0xffffffffu, sl, o);
    if (tid == 0) P.logdet_part[part] = sl;
  }
}

}  // namespace fgpu
