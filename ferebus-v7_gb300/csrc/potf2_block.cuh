// The W x W diagonal-block Cholesky (FP64) with its log-det part, as a
// block-level device routine for W * 4 threads (W / 8 warps): called by its
// own kernel (barrier 0 = the whole CTA) and by the tensor-core coupling
// kernel, whose epilogue warps 0-3 factor the next quarter's diagonal block
// as soon as the tile holding it is coupled (barrier 2).
//
// Right-looking, one column per step, the block held in registers: warp w
// owns the columns c = w + NWARP * k (k < 8), lane l holds rows l + 32 h of
// them.  Step j: the owner of column j has published L(:, j) in a shared ring
// slot and arrived on that slot's mbarrier (a producer-only signal, so no
// warp waits for another's trailing work); every warp subtracts L(r, j) L(c,
// j) from its columns c > j, the owner of column j + 1 first, which then
// takes the pivot of j + 1 (rsqrt, one FP64 multiply per entry) and publishes
// column j + 1 before finishing its other columns.  On this GPU a dependent
// FP64 operation costs ~65 cycles and sqrt + division ~1100, so the critical
// path is one rsqrt (~380 cycles), three dependent FP64 operations and the
// hand-over between warps (~100 cycles) per column: ~1000 cycles, half the
// blocked left-looking form's.  The ring has NWARP + 1 slots: the owner of
// column j + NWARP + 1, which overwrites column j's slot, has by then waited
// for columns j + 1 .. j + NWARP, each published after its owner had read
// column j.  The result differs from dpotf2's (lapack/dpotf2.f) only in the
// order of its sums and in sqrt / division by the pivot being d * rsqrt(d) /
// multiplication by rsqrt(d).  A non-positive pivot sets the problem's
// LAPACK-style info (1-based column) and failed flag; a wait that runs out
// sets the timeout status.
#pragma once
#include "fgpu_internal.h"
#include "tc_common.cuh"

namespace fgpu {

template <int W>
struct PotfShared {
  static constexpr int NSLOT = W / 8 + 1;
  double col[NSLOT][W];     // published columns of L (rows > j)
  uint64_t full[NSLOT];     // one mbarrier per slot, 32 arrivals (the owner warp)
  double diag[W];           // L_cc for the log-det part
  int fail_col;
};

__device__ __forceinline__ void bar_sync_n(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Pivot of column jc by its owner warp: L_jj = d rsqrt(d), L(r, j) =
// a(r, j) rsqrt(d) for r > j; publish the column and arrive on its slot.
// Returns false (after arriving, with fail_col set) for a non-positive pivot.
template <int W, int R, int jc>
__device__ __forceinline__ bool potf2_pivot(double (&a)[8][R], int lane, PotfShared<W>& sh) {
  constexpr int NWARP = W / 8, NSLOT = PotfShared<W>::NSLOT;
  constexpr int kc = jc / NWARP, hd = jc / 32;
  const double d = __shfl_sync(0xffffffffu, a[kc][hd], jc % 32);
  const bool ok = d > 0.0;  // the same in every lane
  if (ok) {
    const double rd = rsqrt(d);
#pragma unroll
    for (int h = 0; h < R; ++h) {
      const int r = lane + 32 * h;
      if (r > jc) {
        a[kc][h] *= rd;
        sh.col[jc % NSLOT][r] = a[kc][h];
      } else if (r == jc) {
        a[kc][h] = d * rd;
        sh.diag[jc] = a[kc][h];
      }
    }
  } else if (lane == 0) {
    sh.fail_col = jc;
  }
  mbar_arrive(&sh.full[jc % NSLOT]);  // release: this lane's stores above
  return ok;
}

// Step j of the factorisation (all warps), then step j + 1: wait for column
// j, subtract it from the warp's columns c > j (the owner of column j + 1
// first, which then pivots), stop on a failed pivot or a wait that ran out.
// Compile-time j keeps a[][] in registers.
template <int W, int R, int j>
__device__ __forceinline__ void potf2_steps(double (&a)[8][R], const Prob& P, int lane, int w, PotfShared<W>& sh,
                                            bool& stop) {
  if constexpr (j < W - 1) {
    constexpr int NWARP = W / 8, NSLOT = PotfShared<W>::NSLOT;
    if (!stop) {  // warp-uniform
      if (!mbar_wait(&sh.full[j % NSLOT], (uint32_t)((j / NSLOT) & 1))) {
        atomicExch(&P.status[2], 1);
        stop = true;
      } else if (*(volatile int*)&sh.fail_col >= 0) {
        stop = true;
      } else {
        double lr[R], lc[8];
#pragma unroll
        for (int h = 0; h < R; ++h) lr[h] = sh.col[j % NSLOT][lane + 32 * h];  // rows <= j: stale, only reach r < c
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int c = w + NWARP * k;
          lc[k] = c > j ? sh.col[j % NSLOT][c] : 0.0;
        }
        constexpr int j1 = j + 1, k1 = j1 / NWARP;
        if (w == j1 % NWARP) {  // owner of the next pivot: its column first
#pragma unroll
          for (int h = 0; h < R; ++h) a[k1][h] = fma(-lr[h], lc[k1], a[k1][h]);
          stop = !potf2_pivot<W, R, j1>(a, lane, sh);
        }
        if (!stop) {
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int c = w + NWARP * k;
            if (c > j1)
#pragma unroll
              for (int h = 0; h < R; ++h) a[k][h] = fma(-lr[h], lc[k], a[k][h]);
          }
        }
      }
    }
    potf2_steps<W, R, j + 1>(a, P, lane, w, sh, stop);
  }
}

template <int W>
__device__ __forceinline__ void potf2_block(const Prob& P, int col0, int part, int tid, PotfShared<W>& sh, int bar) {
  constexpr int NT = W * 4;
  constexpr int NWARP = W / 8;
  constexpr int R = W / 32;  // rows per lane
  constexpr int NSLOT = PotfShared<W>::NSLOT;
  const int lane = tid & 31, w = tid >> 5;
  const size_t ld = (size_t)P.ld;
  double* Kd = P.K + (size_t)col0 * ld + col0;
  double a[8][R];
#pragma unroll
  for (int k = 0; k < 8; ++k)
#pragma unroll
    for (int h = 0; h < R; ++h) {
      const int c = w + NWARP * k, r = lane + 32 * h;
      a[k][h] = r >= c ? Kd[(size_t)c * ld + r] : 0.0;
    }
  if (tid == 0) {
    sh.fail_col = -1;
    for (int s = 0; s < NSLOT; ++s) mbar_init(&sh.full[s], 32);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  bar_sync_n(bar, NT);
  bool stop = false;
  if (w == 0) stop = !potf2_pivot<W, R, 0>(a, lane, sh);
  potf2_steps<W, R, 0>(a, P, lane, w, sh, stop);
  bar_sync_n(bar, NT);
  if (tid == 0)
    for (int s = 0; s < NSLOT; ++s) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(su32(&sh.full[s])) : "memory");
  if (sh.fail_col >= 0) {
    if (tid == 0) {
      P.status[0] = col0 + sh.fail_col + 1;  // LAPACK info: 1-based column
      P.status[1] = 1;
    }
    return;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k)
#pragma unroll
    for (int h = 0; h < R; ++h) {
      const int c = w + NWARP * k, r = lane + 32 * h;
      if (r >= c) Kd[(size_t)c * ld + r] = a[k][h];
    }
  // log-det partial: 2 * sum log(L_jj) is formed in the epilogue
  // (arith.f90:72-93); here the block's sum of logs, in column order.
  if (tid < 32) {
    double sl = 0.0;
    for (int c = tid * (W / 32); c < (tid + 1) * (W / 32); ++c) sl += log(sh.diag[c]);
    for (int o = 16; o > 0; o >>= 1) sl += __shfl_down_sync(0xffffffffu, sl, o);
    if (tid == 0) P.logdet_part[part] = sl;
  }
}

}  // namespace fgpu
