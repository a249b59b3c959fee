// Kernel-matrix build on the tensor cores (tensor-core mode, kernels whose
// leaves are rbf, periodic, linear or constant with at most two rbf/periodic
// leaves).
//
// Both rbf and periodic leaves are exp(-|f_i - f_j|^2 / 2) of a per-leaf
// feature vector: f = sqrt(l) (x - mean) for rbf (stationary_kernel.f90:
// 101-122), f = (cos x, sin x) / exp(theta) per dimension for periodic
// (periodic_kernel.f90:181-206, since 2 sin^2(d/2) = 1 - cos d).  The
// squared distance is formed exactly in integers:
//
//  * Each leaf gets a power-of-two scale 2^s >= max |f| (from the per-plane
//    maxima of |x|, so it needs no reduction); f 2^-s is rounded to 55
//    fractional bits and split into 7 signed base-256 digits, one fp16 plane
//    per digit, written into the (otherwise idle) digit-plane buffer of the
//    factorisation at k offset koff.
//  * tcgen05.mma kind::f16 over the leaf's k range gives 8 exact level sums
//    S_L, L = p + q <= 7, of <f_i, f_j> (the same exactness argument as the
//    trailing update: at most 7 pairs x 128 terms x 129^2 < 2^24).  With
//    f 2^-s = sum_p d_p 2^(-7 - 8p), sum_L S_L 2^(56 - 8L) = <f_i, f_j>
//    2^(70 - 2s) up to the dropped levels L > 7 (below 2^-54 of 2^2s, under
//    the digits' own rounding), which the epilogue rounds to
//    W_ij = <f_i, f_j> 2^(u - 2 - 2s) (u = 60 - ceil(log2 nf): 4 max W < 2^61).
//    The 8 levels of a 128 x 64 tile fill the 512 TMEM columns.
//  * E = W_ii + W_jj - 2 W_ij (W_ii from the same digits, computed
//    exactly when the digits are written) is |f_i - f_j|^2 2^(u - 2 - 2s):
//    zero on the diagonal, and exp(-E 2^(2s + 1 - u)) is evaluated by the
//    fixed-point exponential straight from the integer (the leaf-scale form
//    iexp_fixed_tab: a fixed binary point, two 1024-entry tables in shared
//    memory, a degree-2 polynomial).
//
// The leaf values combine through the kernel expression, which is
// multilinear in the (at most two) distance leaves: k = a + b v0 + c v1 +
// d v0 v1, with a..d from the constant / linear leaves (one thread per
// problem, before the build).  The persistent kernel has the update's
// structure: TMA producer warp, MMA warp, 16 epilogue warps (the epilogue's
// integer work is what bounds the kernel, so it gets the warps); one pass per
// distance leaf per 128 x 64 tile, the first leaf's values kept in shared
// memory for the second pass.  FP64 instructions run at 2 lanes per cycle
// per SM on this part (FP32: 128), so the entry loop holds none but the one
// add of a two-leaf sum: the combination is chosen once per pass, and the
// nugget goes onto the one diagonal entry afterwards.
#include "../../include/fgpu.h"
#include "fgpu_internal.h"
#include "iexp.cuh"
#include "tc_common.cuh"

#include <cmath>

namespace fgpu {

namespace {

// per-plane feature scale of leaf L: rbf sqrt(exp(theta)), periodic 1/exp(theta)
__device__ __forceinline__ double plane_weight(const Leaf& L, const double* theta, int k) {
  return L.type == L_RBF ? exp(0.5 * theta[L.param0 + k]) : 1.0 / exp(theta[L.param0 + k]);
}

// s with max_k |w_k x_ik| < 2^s over every point (from the per-plane maxima)
__device__ __forceinline__ int leaf_scale(const Prob& P, const Leaf& L) {
  const int nf = L.type == L_PERIODIC ? 2 * L.n : L.n;
  double m = 0.0;
  for (int k = 0; k < nf; ++k) {
    const int dim = L.type == L_PERIODIC ? k / 2 : k;
    m = fmax(m, plane_weight(L, P.theta, dim) * P.plane_max[L.plane0 + k]);
  }
  if (m == 0.0) return 0;
  return (int)((__double_as_longlong(m) >> 52) & 0x7FF) - 1022;
}

constexpr int NLEV = 8;  // digit-pair levels p + q = 0..7

// W = round(sum_L S_L 2^(u - 16 - 8L)) from the 8 exact level sums (48 <= u <= 63)
__device__ __forceinline__ long long assemble_w(const int S[NLEV], int u) {
  const long long H = (long long)S[0] * (1LL << 32) + (long long)S[1] * (1LL << 24) + (long long)S[2] * 65536 +
                      (long long)S[3] * 256 + S[4];
  const long long Lo = (long long)S[5] * 65536 + (long long)S[6] * 256 + S[7];
  return (long long)((unsigned long long)H << (u - 48)) + ((Lo + (1LL << (71 - u))) >> (72 - u));
}

// The same W from the magic-add bits b_L = 0x4B400000 + S_L of level sums
// with |S_L| < 2^22 (level_bits): adjacent levels pair up in 32 bits
// (b_L 256 + b_(L+1) = (S_L + 2^22) 256 + (S_(L+1) + 2^22) + 0x4B000000 <
// 2^32, the top byte of b_L leaving modulo 2^32) and the offsets leave as two
// constants, one for the top five levels and one for the last three.
constexpr long long BUILD_BIAS_H = (1LL << 22) * 0x0101010101LL + 0x4B000000LL * ((1LL << 24) + (1LL << 8) + 1);
constexpr long long BUILD_BIAS_LO = (1LL << 22) * 0x010101LL + 0x4B000000LL * ((1LL << 8) + 1);
__device__ __forceinline__ long long assemble_w_bits(const uint32_t b[NLEV], int u) {
  const uint32_t p01 = b[0] * 256u + b[1];
  const uint32_t p23 = b[2] * 256u + b[3];
  const uint32_t p56 = b[5] * 256u + b[6];
  const long long H = (long long)(((unsigned long long)p01 << 24) + ((unsigned long long)p23 << 8) + b[4]) -
                      BUILD_BIAS_H;  // sum_{L<=4} S_L 256^(4-L)
  const long long Lo = (long long)(((unsigned long long)p56 << 8) + b[7]) - BUILD_BIAS_LO;
  return (long long)((unsigned long long)H << (u - 48)) + ((Lo + (1LL << (71 - u))) >> (72 - u));
}

}  // namespace

// ---------------------------------------------------------------------------
// feature digits and exact self dot products; one thread per point
// grid (nt128, nprob) x 128 threads
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_feat_digits(const Prob* __restrict__ probs) {
  const Prob& P = probs[blockIdx.y];
  const int rb = blockIdx.x;
  if (P.mode != 1 || rb >= P.nt128) return;
  const Spec& sp = *P.spec;
  if (!sp.tc_build) return;
  const int r = threadIdx.x, i = rb * NB + r;
  const size_t nc = (size_t)P.Nc;
  __shared__ int s_e[2];
  if (r < sp.ndot) {
    s_e[r] = leaf_scale(P, sp.leaf[sp.dot_leaf[r]]);
    if (rb == 0) P.fscale[r] = s_e[r];
  }
  __syncthreads();
  bool bad = false;
  for (int t = 0; t < sp.ndot; ++t) {
    const Leaf& L = sp.leaf[sp.dot_leaf[t]];
    const int nf = L.type == L_PERIODIC ? 2 * L.n : L.n;
    const int e = s_e[t];
    int S[NLEV] = {0, 0, 0, 0, 0, 0, 0, 0};
    unsigned char* base = P.slices + (size_t)rb * NSLICE * SLICE_BYTES + (size_t)r * 16;
    for (int kg = 0; kg < sp.dot_kch[t] * 2; ++kg) {
      int d[NSLICE][8];
      for (int kk = 0; kk < 8; ++kk) {
        const int k = kg * 8 + kk;
        const double x = (k < nf) ? P.splanes[(size_t)(L.plane0 + k) * nc + i] : 0.0;
        long long F = to_fixed55(x, e, &bad);
        for (int p = NSLICE - 1; p >= 1; --p) {
          const int b = (int)(signed char)(F & 0xFF);
          d[p][kk] = b;
          F = (F - b) >> 8;
        }
        d[0][kk] = (int)F;
        for (int p = 0; p < NSLICE; ++p)
          for (int q = 0; q < NSLICE && p + q < NLEV; ++q) S[p + q] += d[p][kk] * d[q][kk];
      }
      const int kgl = sp.dot_koff[t] / 8 + kg;
      for (int p = 0; p < NSLICE; ++p) {
        __align__(16) __half h[8];
        for (int kk = 0; kk < 8; ++kk) h[kk] = __int2half_rn(d[p][kk]);
        *reinterpret_cast<uint4*>(base + (size_t)p * SLICE_BYTES + (size_t)kgl * 2048) =
            *reinterpret_cast<const uint4*>(h);
      }
    }
    P.fnorm[(size_t)t * nc + i] = assemble_w(S, sp.dot_u[t]);
  }
  if (bad) atomicOr(&P.status[3], 1);
  // multilinear coefficients of the kernel expression in the distance leaves
  if (rb == 0 && r == 0) {
    double stk[MAX_POST][4];
    int top = 0;
    for (int tk = 0; tk < sp.npost; ++tk) {
      const int tok = sp.post[tk];
      if (tok >= 0) {
        const Leaf& L = sp.leaf[tok];
        double c[4] = {0.0, 0.0, 0.0, 0.0};
        if (L.type == L_RBF || L.type == L_PERIODIC) {
          c[tok == sp.dot_leaf[0] ? 1 : 2] = 1.0;
        } else if (L.type == L_LINEAR) {
          // linear_kernel.f90:70-76, order 0: sum_k 1 / exp(-theta_k)
          double a = 0.0;
          for (int k = 0; k < L.n; ++k) a += 1.0 / exp(-P.theta[L.param0 + k]);
          c[0] = a;
        } else {
          c[0] = P.theta[L.param0];  // constant.f90:62-68
        }
        for (int q = 0; q < 4; ++q) stk[top][q] = c[q];
        ++top;
      } else {
        const double* b = stk[--top];
        double* a = stk[top - 1];
        if (tok == P_SUM) {
          for (int q = 0; q < 4; ++q) a[q] += b[q];
        } else {  // each leaf occurs once: no squared terms
          const double c0 = a[0] * b[0];
          const double c1 = a[0] * b[1] + a[1] * b[0];
          const double c2 = a[0] * b[2] + a[2] * b[0];
          const double c3 = a[0] * b[3] + a[3] * b[0] + a[1] * b[2] + a[2] * b[1];
          a[0] = c0;
          a[1] = c1;
          a[2] = c2;
          a[3] = c3;
        }
      }
    }
    for (int q = 0; q < 4; ++q) P.fcoef[q] = stk[0][q];
  }
}

// ---------------------------------------------------------------------------
// persistent tensor-core build of the lower triangle (128 x 64 tiles)
// ---------------------------------------------------------------------------
constexpr int BLD_EPI_WARPS = 16;                      // 4 lane quarters x 4 groups of 16 columns
constexpr int BLD_THREADS = (BLD_EPI_WARPS + 2) * 32;  // + TMA warp + MMA warp
constexpr int NSTAGE = 3;
constexpr uint32_t BLD_TAB = NSTAGE * STAGE + 256;    // the exponential's two tables (2 x 1024 x 8 B)
constexpr uint32_t BLD_STASH = BLD_TAB + 2 * 1024 * 8;  // the first leaf's 16 values per epilogue thread
constexpr uint32_t BLD_SMEM = BLD_STASH + BLD_EPI_WARPS * 32 * 16 * 8;
static_assert(BLD_SMEM <= 227 * 1024, "shared memory per CTA");

__global__ void __launch_bounds__(BLD_THREADS, 1)
    k_build_tc(const Prob* __restrict__ probs, int nprob, const unsigned long long* __restrict__ tiles, int total) {
  extern __shared__ __align__(1024) unsigned char smb[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smb + NSTAGE * STAGE);
  uint64_t* empty = full + NSTAGE;
  uint64_t* tfull = full + 2 * NSTAGE;
  uint64_t* tempty = tfull + 1;
  uint64_t* drain = tfull + 2;  // quiescing after a give-up
  uint32_t* slot = reinterpret_cast<uint32_t*>(tfull + 3);
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint32_t issued = 0;  // producer lane: k-chunks whose operand copies were issued
  if (tid == 0) {
    s_abort = 0;
    mbar_init(drain, 1);
    for (int k = 0; k < NSTAGE; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, BLD_EPI_WARPS * 32);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == BLD_EPI_WARPS + 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = *slot;
  unsigned long long* tab = reinterpret_cast<unsigned long long*>(smb + BLD_TAB);
  unsigned long long* fine = tab + 1024;
  double* stash = reinterpret_cast<double*>(smb + BLD_STASH);
  for (int k = tid; k < 1024; k += BLD_THREADS) {
    tab[k] = g_iexp_tab1024[k];
    fine[k] = g_iexp_fine1024[k];
  }
  __syncthreads();
  // tile t: (problem << 40 | 128-row tile << 20 | 64-column tile), host-built
  auto tile_of = [&](int t, int& p, int& ti, int& tj) {
    const unsigned long long e = tiles[t];
    p = (int)(e >> 40);
    ti = (int)((e >> 20) & 0xFFFFF);
    tj = (int)(e & 0xFFFFF);
  };

  if (warp == BLD_EPI_WARPS) {
    // ---------------- TMA producer: digit planes of each leaf's k chunks ----------------
    if (lane == 0) {
      uint32_t g = 0;
      for (int t = blockIdx.x; t < total && !s_abort; t += gridDim.x) {
        int p, ti, tj;
        tile_of(t, p, ti, tj);
        const Prob& P = probs[p];
        const Spec& sp = *P.spec;
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(P.tmap_a) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(P.tmap_b) : "memory");
        for (int d = 0; d < sp.ndot; ++d) {
          const int c0 = sp.dot_koff[d] / 16;
          for (int c = 0; c < sp.dot_kch[d]; ++c, ++g) {
            const int st = g % NSTAGE;
            if (!mbar_wait(&empty[st], ((g / NSTAGE) & 1) ^ 1)) {
              s_abort = 1;
              break;
            }
            unsigned char* As = smb + st * STAGE;
            mbar_expect_tx(&full[st], STAGE);
            tma_load_5d(As, P.tmap_a, 0, 0, 2 * (c0 + c), 0, ti, &full[st]);
            tma_load_5d(As + A_STAGE, P.tmap_b, 0, (tj & 1) * 2, 2 * (c0 + c), 0, tj >> 1, &full[st]);
            issued = g + 1;
          }
          if (s_abort) break;
        }
      }
    }
  } else if (warp == BLD_EPI_WARPS + 1) {
    // ---------------- MMA issuer: one pass of 35 pairs per chunk per leaf ----------------
    if (lane == 0) {
      uint32_t g = 0, it = 0;
      const uint64_t adesc0 = smem_desc(su32(smb), 2048, 128);
      const uint64_t bdesc0 = smem_desc(su32(smb) + A_STAGE, 1024, 128);
      for (int t = blockIdx.x; t < total && !s_abort; t += gridDim.x) {
        int p, ti, tj;
        tile_of(t, p, ti, tj);
        const Spec& sp = *probs[p].spec;
        for (int d = 0; d < sp.ndot; ++d, ++it) {
          if (!mbar_wait(tempty, (it & 1) ^ 1)) {
            s_abort = 1;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          for (int c = 0; c < sp.dot_kch[d]; ++c, ++g) {
            const int st = g % NSTAGE;
            if (!mbar_wait(&full[st], (g / NSTAGE) & 1)) {
              s_abort = 1;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint64_t soff = (uint64_t)((st * STAGE) >> 4);
#pragma unroll
            for (int pp = 0; pp < NSLICE; ++pp) {
#pragma unroll
              for (int q = 0; q < NSLICE && q + pp < NLEV; ++q) {
                // the first pair of level L = pp + q is (max(0, L - 6), .): it starts the sum
                const bool first = c == 0 && pp == (pp + q > NSLICE - 1 ? pp + q - (NSLICE - 1) : 0);
                mma_f16(tbase + (uint32_t)(pp + q) * 64, adesc0 + soff + (uint64_t)(pp * 4096 >> 4),
                        bdesc0 + soff + (uint64_t)(q * 2048 >> 4), first ? 0u : 1u);
              }
            }
            mma_commit(&empty[st]);
          }
          if (s_abort) break;
          mma_commit(tfull);
        }
      }
    }
  } else {
    // ---------------- epilogue (warps 0-15) ----------------
    const int r = (warp & 3) * 32 + lane;  // TMEM lane = tile row
    const int h = warp >> 2;               // group of 16 columns
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t it = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
      int p, ti, tj;
      tile_of(t, p, ti, tj);
      const Prob& P = probs[p];
      const Spec& sp = *P.spec;
      const size_t nc = (size_t)P.Nc;
      const int i = ti * NB + r;
      const int j0 = tj * TB + h * 16;
      bool stop = false;
      for (int d = 0; d < sp.ndot; ++d, ++it) {
        if (!mbar_wait(tfull, it & 1)) {
          s_abort = 1;
          stop = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        long long W[16];
        const int u = sp.dot_u[d];
        // level sums of a leaf with at most 36 features stay below 2^22 (7
        // digit pairs x 36 terms x 2^14): converted by the exact magic add
        // (one FP32 add each, no conversion instruction), otherwise by F2I
        const Leaf& LF = sp.leaf[sp.dot_leaf[d]];
        const bool small = (LF.type == L_PERIODIC ? 2 * LF.n : LF.n) <= 36;
#pragma unroll
        for (int gq = 0; gq < 2; ++gq) {
          uint32_t v[NLEV][8];
#pragma unroll
          for (int l = 0; l < NLEV; ++l) {
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(v[l][0]), "=r"(v[l][1]), "=r"(v[l][2]), "=r"(v[l][3]), "=r"(v[l][4]),
                           "=r"(v[l][5]), "=r"(v[l][6]), "=r"(v[l][7])
                         : "r"(tbase + lane_base + (uint32_t)(l * 64 + h * 16 + gq * 8)));
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;");
          if (small) {
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
              uint32_t b[NLEV];
#pragma unroll
              for (int l = 0; l < NLEV; ++l) b[l] = level_bits(v[l][jj]);
              W[gq * 8 + jj] = assemble_w_bits(b, u);
            }
          } else {
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) {
              int S[NLEV];
#pragma unroll
              for (int l = 0; l < NLEV; ++l) S[l] = __float2int_rn(__uint_as_float(v[l][jj]));
              W[gq * 8 + jj] = assemble_w(S, u);
            }
          }
        }
        // TMEM drained: the next pass's MMAs may start
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(tempty);
        const IexpScale esc = iexp_scale(2 * P.fscale[d] + 1 - u);
        const long long wi = P.fnorm[(size_t)d * nc + i];
        // W_jj of this thread's 16 columns (the same for the whole warp), two at a time
        const longlong2* wj2 = reinterpret_cast<const longlong2*>(P.fnorm + (size_t)d * nc + j0);
        // The combination of the leaf values is chosen once per pass, outside
        // the entry loop: a ternary inside it is compiled into both sides,
        // and every FP64 operation costs this part's narrow FP64 pipe.  A
        // plain sum of the two leaves (a = d = 0, b = c = 1) is one add, the
        // same double as the general form.
        const double ca = P.fcoef[0], cb = P.fcoef[1], cc = P.fcoef[2], cd = P.fcoef[3];
        const int N = P.N;
        double* K = P.K;
        const size_t ld = (size_t)P.ld;
        double kdiag = 0.0;  // this row's diagonal entry, when the tile holds it
        // entry (i, j0 + q): lower triangle of the N x N block; identity padding
        auto put = [&](int q, double kv) {
          const int j = j0 + q;
          if (j == i) kdiag = kv;
          K[(size_t)j * ld + i] = (j > i || i >= N || j >= N) ? (i == j ? 1.0 : 0.0) : kv;
        };
        auto leaf = [&](int q) {
          const longlong2 w2 = __ldg(wj2 + q / 2);
          long long E = wi + ((q & 1) ? w2.y : w2.x) - 2 * W[q];
          E = E < 0 ? 0 : E;
          return iexp_fixed_tab((unsigned long long)E, esc, tab, fine);
        };
        double* st = stash + tid;  // the first leaf's values, for the second pass
        if (d < sp.ndot - 1) {
#pragma unroll
          for (int q = 0; q < 16; ++q) st[q * (BLD_EPI_WARPS * 32)] = leaf(q);
        } else if (d == 0 && cb == 1.0 && ca == 0.0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) put(q, leaf(q));
        } else if (d == 0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) put(q, fma(cb, leaf(q), ca));
        } else if (ca == 0.0 && cb == 1.0 && cc == 1.0 && cd == 0.0) {
#pragma unroll
          for (int q = 0; q < 16; ++q) put(q, st[q * (BLD_EPI_WARPS * 32)] + leaf(q));
        } else {
#pragma unroll
          for (int q = 0; q < 16; ++q) {
            // second distance leaf: k = (d v0 + c) v1 + (b v0 + a)
            const double v0 = st[q * (BLD_EPI_WARPS * 32)];
            put(q, fma(fma(cd, v0, cc), leaf(q), fma(cb, v0, ca)));
          }
        }
        // the nugget on the diagonal (the loop stored the entry without it)
        if (d == sp.ndot - 1 && i >= j0 && i < j0 + 16 && i < N) {
          const double noise = P.optimise_noise ? P.theta[sp.nkparams] : P.noise;
          K[(size_t)i * ld + i] = kdiag + noise * 1.0;
        }
      }
      if (stop) break;
    }
  }
  __syncthreads();
  if (s_abort) {
    // a bounded wait gave up: the copies and MMAs this CTA issued finish
    // (bounded waits) before it frees its TMEM and exits
    if (warp == BLD_EPI_WARPS && lane == 0) drain_ring(full, NSTAGE, issued);
    if (warp == BLD_EPI_WARPS + 1 && lane == 0) drain_mmas(drain);
    __syncthreads();
    if (tid == 0)
      for (int q = 0; q < nprob; ++q) atomicExch(&probs[q].status[2], 1);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == BLD_EPI_WARPS + 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase));
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
cudaError_t launch_feat_digits(const Prob* probs, int nprob, int max_nt128, cudaStream_t s) {
  k_feat_digits<<<dim3(max_nt128, nprob), 128, 0, s>>>(probs);
  return cudaGetLastError();
}

cudaError_t launch_build_tc(const Prob* probs, int nprob, const unsigned long long* tiles, int total_tiles,
                            int num_sms, cudaStream_t s) {
  cudaError_t e = ensure_smem_attr((const void*)k_build_tc, SMEM_BUILD_TC, BLD_SMEM);
  if (e != cudaSuccess) return e;
  if (total_tiles <= 0) return cudaSuccess;
  const int grid = total_tiles < num_sms ? total_tiles : num_sms;
  k_build_tc<<<grid, BLD_THREADS, BLD_SMEM, s>>>(probs, nprob, tiles, total_tiles);
  return cudaGetLastError();
}

}  // namespace fgpu
