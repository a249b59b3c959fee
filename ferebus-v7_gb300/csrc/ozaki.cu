// Tensor-core trailing update for the FP64 Cholesky (mode 1).
//
// GB300 executes FP64 at about 1.1 TFLOP/s, so the O(N^3) trailing update is
// moved to the 5th-generation tensor cores as an exact integer computation
// (the error-free splitting of Ozaki, Ogita and Oishi, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012, with the
// power-of-two row scaling of its tensor-core use by Mukunoki et al., 2020):
//
//  * Row i of the factor has a FIXED power-of-two scale 2^e_i >= sqrt(K_ii):
//    since sum_k L_ik^2 = K_ii, every |L_ik| <= 2^e_i for all panels.
//  * L_ik 2^-e_i is rounded to 55 fractional bits and written as 7 signed
//    base-256 digits d_0..d_6 (|d| <= 129), one fp16 plane per digit.
//  * For a 128-wide panel, digit planes p (rows i) and q (rows j) are
//    multiplied by tcgen05.mma kind::f16 with f32 accumulation.  Products
//    are exact (|d_p d_q| < 2^15) and every partial sum of one level
//    L = p + q (at most 7 pairs x 128 terms x 129^2 < 2^24) is an exact
//    integer in f32, so the 7 level accumulators in TMEM hold exact integers.
//    Levels p + q > 6 (weights below 2^-62 of the row scales) are dropped.
//  * The epilogue turns the 7 exact level sums into one int64 and ADDS it
//    to a per-element integer accumulator in HBM (every partial sum of
//    L_ik L_jk is below 2^(e_i + e_j) by Cauchy-Schwarz, i.e. below 2^62 in
//    the accumulator's units, so 64 bits hold it exactly): the trailing
//    matrix update is exact integer arithmetic, order independent, and uses
//    no FP64 instruction.  When a block column becomes the next panel, one
//    FP64 conversion per element subtracts the accumulated sum from K.
//
// The diagonal 128 x 128 factor, the panel solve and the right-hand-side
// (border) rows stay in FP64.
#include "fgpu_internal.h"
#include "tc_common.cuh"
#include "potf2_block.cuh"

#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>

namespace fgpu {

// ---------------------------------------------------------------------------
// per-row scales from the diagonal of K
// ---------------------------------------------------------------------------
__global__ void k_scales(const Prob* __restrict__ probs) {
  const Prob& P = probs[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (P.mode != 1 || i >= P.Nc) return;
  const double d = P.K[(size_t)i * P.ld + i];
  int e = 0;
  if (d > 0.0 && d < 1e300) {
    int E;
    frexp(sqrt(d) * (1.0 + 0x1p-20), &E);  // sqrt(K_ii) (1 + 2^-20) < 2^E
    e = E;
  }
  P.escale[i] = e;
  P.pw2[i] = ldexp(1.0, e - 31);
}

// ---------------------------------------------------------------------------
// block column s: K_ij -= W_ij 2^(e_i + e_j - 62), rows [c0, Nc)
// ---------------------------------------------------------------------------
constexpr int PP_COLS = 4;  // columns per thread of the panel conversion (a 64-column tile holds 16 groups)
static_assert(8 % PP_COLS == 0, "a thread's columns stay inside one 8-column group of an accumulator piece");
__global__ void __launch_bounds__(256) k_panel_prep(const Prob* __restrict__ probs, int s) {
  const Prob& P = probs[blockIdx.z];
  if (P.mode != 1 || s >= P.nt128 || s == 0 || P.status[1]) return;
  const int c0 = s * NB;
  const int i = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.Nc) return;
  const size_t ld = (size_t)P.ld;
  const int ei = P.escale[i] - 62;
  // PP_COLS columns per thread, their loads issued together (the
  // accumulators and K never overlap, which the compiler cannot know)
  const int jb = c0 + blockIdx.y * PP_COLS;  // PP_COLS columns inside one 8-column group of a piece
  const size_t a0 = acc_tile(i >> 7, jb >> 6, P.nt128) * ACC_TILE_ELEMS + acc_elem(i & 127, jb & 63);
  double* kp = P.K + (size_t)jb * ld + i;
  long long w[PP_COLS];
  int ej[PP_COLS];
  double kv[PP_COLS];
#pragma unroll
  for (int jj = 0; jj < PP_COLS; ++jj) {
    w[jj] = P.acc[a0 + (size_t)jj * 32];
    kv[jj] = kp[(size_t)jj * ld];
    ej[jj] = P.escale[jb + jj];
  }
#pragma unroll
  for (int jj = 0; jj < PP_COLS; ++jj)
    kp[(size_t)jj * ld] = kv[jj] - w64_to_double(w[jj], ei + ej[jj]);
}

// ---------------------------------------------------------------------------
// trailing update of the integer accumulators: persistent, warp-specialised
//
// Output tiles are 128 rows x 64 columns; a tile's 7 level sums occupy 448
// TMEM columns.  Warp 16 (one lane) streams the digit planes of each
// k-chunk of 16 by 5-D TMA into a 4-stage ring; warp 17 (one lane) issues
// the chunk's 28 digit pairs as 10 tcgen05.mma with B's planes stacked
// along N (upd_issue_chunk); warps 0-15 drain TMEM into registers (16
// columns per thread, two rounds of TMEM loads), release it (so the next
// tile's MMAs start), then stage each 8-column piece of the tile's exact
// sums (2 KB, contiguous in the accumulator layout) in shared memory and
// add it to the accumulators in HBM with one bulk reduction
// (cp.reduce.async.bulk .add.u64: the L2 adds, exactly, modulo 2^64), while
// the tensor cores work on the next tile.  The accumulators never pass
// through the SM, which leaves the shared memory to a fourth operand stage.
// (Per-element 64-bit reductions instead, with a fifth stage in the freed
// staging memory, measured slower: the L2 takes them at about half the
// bulk path's rate.)
//
// Accumulator per element: W (int64), value W * 2^(e_i + e_j - 62);
// |W| < 2^62 (see above); tile-major storage of the lower
// triangle's 128 x 64 tiles (acc_tile), column-major inside.  Tiles of a
// step are enumerated problem by problem (a packed list from the host),
// column tile major, row tile minor.
// ---------------------------------------------------------------------------
constexpr int CH = 8;                                // k-chunks of 16 per 128-panel (one MMA each)
constexpr int NSTAGE = 4;
constexpr uint32_t UPD_PIECE = 8 * 32 * 8;  // one warp's staged accumulator piece: 8 columns x 32 rows (2 KB)
constexpr int UPD_MMA_WARPS = 1;  // the epilogue's conversion below takes all 7 levels of a column group at once
// epilogue warps: 4 TMEM lane quarters x UPD_EPI_WARPS / 4 column groups; the
// tile's 7 levels drain in 64 / (UPD_EPI_WARPS / 4) / 8 rounds of 8 columns
// per thread, and the next tile's MMAs wait for the last round
constexpr int UPD_EPI_WARPS = 16;
constexpr int UPD_COLS = 64 / (UPD_EPI_WARPS / 4);  // columns per epilogue thread
constexpr int UPD_TMA_WARP = UPD_EPI_WARPS, UPD_MMA_WARP = UPD_EPI_WARPS + 1;
constexpr int UPD_THREADS = 32 * (UPD_EPI_WARPS + 1 + UPD_MMA_WARPS);  // epilogue, TMA, MMA issue
static_assert(UPD_COLS % 8 == 0 && UPD_EPI_WARPS % 4 == 0, "epilogue column groups of 8");
constexpr uint32_t UPD_SMEM = NSTAGE * STAGE + UPD_EPI_WARPS * UPD_PIECE + 256;
static_assert(UPD_SMEM <= 227 * 1024, "shared memory per CTA");

// MMA-issuing warp of digit level l (one warp issues all levels)
__host__ __device__ constexpr int upd_level_warp(int) { return 0; }
static_assert(UPD_MMA_WARPS == 1, "the update epilogue converts all 7 levels of a column group in one pass");

// one k-chunk of a tile with the B planes stacked along N: for A plane pp
// the pairs (pp, q), q = 0 .. 6 - pp, accumulate into levels pp .. 6, whose
// TMEM blocks of 64 columns are contiguous, so they are one MMA over B
// planes 0 .. 6 - pp (N = 64 (7 - pp), above N = 256 in two equal halves): 10 MMAs instead of
// 28, and A plane pp is read from shared memory once or twice instead of
// 7 - pp times.  N >= 128 MMAs run at the tensor pipe's full rate; N = 64
// ones are bound by shared-memory operand bandwidth.
__device__ __forceinline__ void upd_issue_chunk(uint32_t tbase, uint64_t adesc, uint64_t bdesc, bool first) {
#pragma unroll
  for (int pp = 0; pp < NSLICE; ++pp) {
    // N = 64 (7 - pp) in one MMA, or, above the 256 limit, in two equal
    // halves (224 + 224, 192 + 192, 160 + 160): an N = 64 remainder would
    // be bound by the A operand's shared-memory read rather than the tensor
    // pipe.  The stacked B rows and the TMEM columns are both contiguous, so
    // a split at any multiple of 8 rows is one offset in each.
    const int n = 64 * (NSLICE - pp);
    const int nh = n <= 256 ? n : n / 2;
#pragma unroll
    for (int off = 0; off < n; off += nh) {
      const uint32_t idesc = (1u << 4) | ((uint32_t)(nh >> 3) << 17) | ((128u >> 4) << 24);
      mma_f16_desc(tbase + (uint32_t)(pp * 64 + off), adesc + (uint64_t)(pp * 4096 >> 4),
                   bdesc + (uint64_t)((off * 16) >> 4), idesc, (first && pp == 0) ? 0u : 1u);
    }
  }
}

__global__ void __launch_bounds__(UPD_THREADS, 1)
    k_ozaki_update(const Prob* __restrict__ probs, int nprob, int s, const unsigned long long* __restrict__ tiles,
                   int total) {
  extern __shared__ __align__(1024) unsigned char smu[];
  unsigned char* pieces = smu + NSTAGE * STAGE;  // [epilogue warp]: its staged accumulator piece
  uint64_t* full = reinterpret_cast<uint64_t*>(smu + NSTAGE * STAGE + UPD_EPI_WARPS * UPD_PIECE);
  uint64_t* empty = full + NSTAGE;
  uint64_t* tfull = full + 2 * NSTAGE;
  uint64_t* tempty = tfull + 1;                     // [UPD_MMA_WARPS]: that warp's levels drained
  uint64_t* drain = tempty + UPD_MMA_WARPS;         // quiescing after a give-up
  uint32_t* slot = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint32_t issued = 0;  // producer lane: k-chunks whose operand copies were issued
  if (tid == 0) {
    s_abort = 0;
    for (int k = 0; k < NSTAGE; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], UPD_MMA_WARPS);  // a commit from each MMA warp
    }
    mbar_init(tfull, UPD_MMA_WARPS);
    for (int k = 0; k < UPD_MMA_WARPS; ++k) mbar_init(&tempty[k], UPD_EPI_WARPS * 32);
    mbar_init(drain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == UPD_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = *slot;
  // tile t of the step: one load instead of a search over the problems
  auto tile_of = [&](int t, int& p, int& ti, int& tj) {
    const unsigned long long e = tiles[t];
    p = (int)(e >> 40);
    ti = (int)((e >> 20) & 0xFFFFF);
    tj = (int)(e & 0xFFFFF);
  };

  if (warp == UPD_TMA_WARP) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      uint32_t g = 0;
      for (int t = blockIdx.x; t < total; t += gridDim.x) {
        int p, ti, tj;
        tile_of(t, p, ti, tj);
        const Prob& P = probs[p];
        if (P.status[1]) continue;
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(P.tmap_a) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(P.tmap_bs) : "memory");
        for (int c = 0; c < CH; ++c, ++g) {
          const int st = g % NSTAGE;
          if (!mbar_wait(&empty[st], ((g / NSTAGE) & 1) ^ 1)) {
            s_abort = 1;
            break;
          }
          unsigned char* As = smu + st * STAGE;
          mbar_expect_tx(&full[st], STAGE);
          tma_load_5d(As, P.tmap_a, 0, 0, 2 * c, 0, ti, &full[st]);
          tma_load_5d(As + A_STAGE, P.tmap_bs, 0, (tj & 1) * 2, 0, 2 * c, tj >> 1, &full[st]);
          issued = g + 1;
        }
        if (s_abort) break;
      }
    }
  } else if (warp >= UPD_MMA_WARP) {
    // ---------------- MMA issue ----------------
    const int mw = warp - UPD_MMA_WARP;
    if (lane == 0) {
      uint32_t g = 0, it = 0;
      const uint64_t adesc0 = smem_desc(su32(smu), 2048, 128);
      const uint64_t bdesc0 = smem_desc(su32(smu) + A_STAGE, NSLICE * 1024, 128);  // [k-group][plane][row]
      for (int t = blockIdx.x; t < total; t += gridDim.x) {
        int p, ti, tj;
        tile_of(t, p, ti, tj);
        if (probs[p].status[1]) continue;
        if (!mbar_wait(&tempty[mw], (it & 1) ^ 1)) {  // this warp's levels of the previous tile drained
          s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        bool ok = true;
        for (int c = 0; c < CH; ++c, ++g) {
          const int st = g % NSTAGE;
          if (!mbar_wait(&full[st], (g / NSTAGE) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t soff = (uint64_t)((st * STAGE) >> 4);
          upd_issue_chunk(tbase, adesc0 + soff, bdesc0 + soff, c == 0);
          mma_commit(&empty[st]);
        }
        if (!ok) {
          s_abort = 1;
          break;
        }
        mma_commit(tfull);
        ++it;
      }
    }
  } else {
    // ---------------- epilogue (warps 0 .. UPD_EPI_WARPS - 1) ----------------
    const int h = warp >> 2;  // column group of UPD_COLS; TMEM lanes (tile rows) 32 (warp & 3) + lane
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t it = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x) {
      int p, ti, tj;
      tile_of(t, p, ti, tj);
      const Prob& P = probs[p];
      if (P.status[1]) continue;
      if (!mbar_wait(tfull, it & 1)) {
        s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      // drain the 7 level sums of this thread's columns in groups of 8;
      // W = sum_l S_l 2^(48 - 8 l) is gathered on the way in unsigned,
      // wrapping arithmetic (partial sums may pass 2^63, the total W stays
      // below 2^62)
      unsigned long long wv[UPD_COLS];
#pragma unroll
      for (int gq = 0; gq < UPD_COLS / 8; ++gq) {
        const int col0 = h * UPD_COLS + gq * 8;
        uint32_t v[NSLICE][8];
#pragma unroll
        for (int l = 0; l < NSLICE; ++l)
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                       : "=r"(v[l][0]), "=r"(v[l][1]), "=r"(v[l][2]), "=r"(v[l][3]), "=r"(v[l][4]),
                         "=r"(v[l][5]), "=r"(v[l][6]), "=r"(v[l][7])
                       : "r"(tbase + lane_base + (uint32_t)(l * 64 + col0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        // Exact integer level sums without the conversion unit (see
        // level_bits) when every sum of the warp's group lies in (-2^22,
        // 2^22) (up to 2^24 in principle, far rarer in practice); otherwise
        // the warp converts this group with F2I.  The range is checked on the
        // raw sums, so the conversion itself needs no second TMEM read and
        // can follow the release below.
        float mx = 0.0f;
#pragma unroll
        for (int l = 0; l < NSLICE; ++l)
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) mx = fmaxf(mx, fabsf(__uint_as_float(v[l][jj])));
        const bool magic = __all_sync(0xffffffffu, mx < 4194304.0f);
        if (gq == UPD_COLS / 8 - 1) {
          // every level sum of the tile is in registers: the next tile's
          // MMAs may overwrite these TMEM columns while the last group converts
          asm volatile("tcgen05.fence::before_thread_sync;");
          mbar_arrive(&tempty[0]);
        }
        if (magic) {
#pragma unroll
          for (int l = 0; l < NSLICE; ++l)
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) v[l][jj] = level_bits(v[l][jj]);
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) wv[gq * 8 + jj] = (unsigned long long)level_bits_to_w64(v, jj);
        } else {
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) {
            int S[NSLICE];
#pragma unroll
            for (int l = 0; l < NSLICE; ++l) S[l] = __float2int_rn(__uint_as_float(v[l][jj]));
            wv[gq * 8 + jj] = (unsigned long long)levels_to_w64(S);
          }
        }
      }
      // each 8-column group of this warp's 32 rows is one contiguous 2 KB
      // piece of the accumulator tile (acc_elem): staged in shared memory,
      // then added to HBM by one bulk reduction from lane 0 (step 0 stores it)
      long long* ga = P.acc + acc_tile(ti, tj, P.nt128) * ACC_TILE_ELEMS;
      unsigned long long* stg = reinterpret_cast<unsigned long long*>(pieces + warp * UPD_PIECE);
#pragma unroll
      for (int pc = 0; pc < UPD_COLS / 8; ++pc) {
        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the last reduction has read the buffer
        __syncwarp();
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) stg[jj * 32 + lane] = wv[pc * 8 + jj];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the bulk copy
        __syncwarp();
        if (lane == 0) {
          long long* dst = ga + acc_elem((warp & 3) * 32, h * UPD_COLS + pc * 8);
          if (s == 0)
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(su32(stg)),
                         "r"(UPD_PIECE)
                         : "memory");
          else
            asm volatile("cp.reduce.async.bulk.global.shared::cta.bulk_group.add.u64 [%0], [%1], %2;" ::"l"(dst),
                         "r"(su32(stg)), "r"(UPD_PIECE)
                         : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
      }
      ++it;
    }
  }
  // the accumulator reductions this warp issued complete before the CTA
  // (and its staged pieces) goes away
  if (warp < UPD_EPI_WARPS && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  __syncthreads();
  if (s_abort) {
    // a bounded wait gave up: before the CTA frees its TMEM and exits, the
    // operand copies it issued land and its MMAs complete (each of these
    // waits is bounded too), then every problem of this step is flagged
    if (warp == UPD_TMA_WARP && lane == 0) drain_ring(full, NSTAGE, issued);
    if (warp == UPD_MMA_WARP && lane == 0) drain_mmas(drain);
    __syncthreads();
    if (tid == 0)
      for (int q = 0; q < nprob; ++q) atomicExch(&probs[q].status[2], 1);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == UPD_MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase));
}

// ---------------------------------------------------------------------------
// coupling inside panel s on the tensor cores: for source quarters
// [sq, sq + ns) and destination quarters [dq, dq + NQ) (32 columns each),
//   K[i, c0+32dq+j] -= sum_{k in source} L[i, c0+k] L[c0+32dq+j, c0+k],
// for rows i >= c0 + 32 dq, from the digit planes of the source quarters.
// The panel uses three: quarter 0 -> 1, half 0 -> half 1, quarter 2 -> 3.
// Persistent and warp-specialised like the trailing update: one lane of
// warp 16 streams the k-chunks of each 128-row tile (A: 128 rows; B: the
// destination's 32 NQ rows) through a 3-stage ring, one lane of warp 17
// issues the MMAs (N = 32 NQ) into TMEM (two buffers of 7 x 32 columns for
// NQ = 1, one of 7 x 64 for NQ = 2), warps 0-15 drain the level sums (warps
// w, w + 4, w + 8, w + 12 share TMEM lanes 32 (w % 4) and take a quarter of
// the columns each, in groups of 8 with the next group's K entries in
// flight; four warps per SMSP hide the integer conversion's latency; a
// warp frees its share of the buffer once the tile's last group is in
// registers, before that group converts) and subtract the exactly
// converted sums from K; warp 18 applies the same
// coupling to the right-hand-side rows in FP64.  Once the epilogue warps have coupled a
// problem's own 128-row tile (barrier 1), warps 0-3 factor quarter dq's
// 32 x 32 diagonal block right there (barrier 2).
// Tiles are handed out dynamically (an atomic counter over a host-built
// order in which every problem's own row tile comes first), so the CTAs
// that factor a diagonal block take correspondingly fewer tiles and the
// factors' FP64 latency hides behind the other CTAs' couplings.  The
// producer lane fetches each tile id and passes it to the MMA and epilogue
// warps through a 4-entry ring in shared memory.
// ---------------------------------------------------------------------------
constexpr int CPL_NSTAGE = 3;
constexpr uint32_t CPL_SMEM = CPL_NSTAGE * STAGE + 256;
constexpr int CPL_EPI_WARPS = 16;                     // 4 TMEM lane quarters x 4 column groups
constexpr int CPL_TMA_WARP = CPL_EPI_WARPS, CPL_MMA_WARP = CPL_EPI_WARPS + 1, CPL_RHS_WARP = CPL_EPI_WARPS + 2;
constexpr int CPL_THREADS = 32 * (CPL_EPI_WARPS + 3);  // epilogue, TMA, MMA, right-hand-side rows
constexpr int CPL_EPI = 32 * CPL_EPI_WARPS;            // epilogue threads

template <int NQ>
__global__ void __launch_bounds__(CPL_THREADS, 1)
    k_couple(const Prob* __restrict__ probs, int nprob, int s, int sq, int ns, int dq,
             const int* __restrict__ order, int total, int* __restrict__ counter) {
  constexpr int N = 32 * NQ;
  constexpr uint32_t B_BYTES = NSLICE * 2 * N * 16;    // 7 planes x 2 k-groups x N rows x 16 B
  constexpr uint32_t CSTAGE = A_STAGE + B_BYTES;
  constexpr int NBUF = NQ == 1 ? 2 : 1;                 // TMEM buffers of 7 N columns
  extern __shared__ __align__(1024) unsigned char smq[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smq + CPL_NSTAGE * STAGE);
  uint64_t* empty = full + CPL_NSTAGE;
  uint64_t* tfull = full + 2 * CPL_NSTAGE;  // [2]
  uint64_t* tempty = tfull + 2;             // [2]
  uint64_t* idf = tfull + 4;                // [4] tile id published
  uint64_t* ide = tfull + 8;                // [4] tile id read by the MMA lane and the epilogue threads
  uint64_t* drain = tfull + 12;             // quiescing after a give-up
  uint32_t* slot = reinterpret_cast<uint32_t*>(tfull + 13);
  __shared__ int s_abort;
  __shared__ int s_tile[4];
  __shared__ PotfShared<QW> s_potf;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nch = 2 * ns;
  uint32_t issued = 0;  // producer lane: k-chunks whose operand copies were issued
  if (tid == 0) {
    s_abort = 0;
    mbar_init(drain, 1);
    for (int k = 0; k < CPL_NSTAGE; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], 1);
    }
    for (int k = 0; k < 2; ++k) {
      mbar_init(&tfull[k], 1);
      mbar_init(&tempty[k], CPL_EPI);
    }
    for (int k = 0; k < 4; ++k) {
      mbar_init(&idf[k], 1);
      mbar_init(&ide[k], CPL_EPI + 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == CPL_MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = *slot;
  // next tile id from the ring (-1: no more tiles); false if the wait gave up
  auto next_tile = [&](uint32_t k, int& id) -> bool {
    const int sl = k & 3;
    if (!mbar_wait(&idf[sl], (k >> 2) & 1)) return false;
    id = *(volatile int*)&s_tile[sl];
    mbar_arrive(&ide[sl]);
    return true;
  };

  if (warp == CPL_TMA_WARP) {
    // ---------------- TMA producer (and tile fetcher) ----------------
    if (lane == 0) {
      uint32_t g = 0;
      for (uint32_t k = 0;; ++k) {
        const int sl = k & 3;
        if (!mbar_wait(&ide[sl], ((k >> 2) & 1) ^ 1)) {
          s_abort = 1;
          break;
        }
        const int u = s_abort ? total : atomicAdd(counter, 1);
        const int id = u < total ? order[u] : -1;
        s_tile[sl] = id;
        mbar_arrive(&idf[sl]);
        if (id < 0) break;
        const int p = id >> 16, ti = id & 0xFFFF;
        const Prob& P = probs[p];
        const void* tb = NQ == 1 ? P.tmap_bs32 : P.tmap_bs;  // planes stacked along N
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(P.tmap_a) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tb) : "memory");
        for (int c = 0; c < nch; ++c, ++g) {
          const int st = g % CPL_NSTAGE;
          if (!mbar_wait(&empty[st], ((g / CPL_NSTAGE) & 1) ^ 1)) {
            s_abort = 1;
            break;
          }
          unsigned char* As = smq + st * STAGE;
          const int kg = 2 * (2 * sq + c);
          mbar_expect_tx(&full[st], CSTAGE);
          tma_load_5d(As, P.tmap_a, 0, 0, kg, 0, ti, &full[st]);
          tma_load_5d(As + A_STAGE, tb, 0, dq, 0, kg, s, &full[st]);  // rows c0+32dq .. +N-1
          issued = g + 1;
        }
      }
    }
  } else if (warp == CPL_MMA_WARP) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      uint32_t g = 0, it = 0;
      const uint64_t adesc0 = smem_desc(su32(smq), 2048, 128);
      const uint64_t bdesc0 = smem_desc(su32(smq) + A_STAGE, NSLICE * N * 16, 128);  // [k-group][plane][row]
      for (uint32_t k = 0;; ++k, ++it) {
        int id;
        if (!next_tile(k, id)) {
          s_abort = 1;
          break;
        }
        if (id < 0) break;
        const int buf = it % NBUF;
        const uint32_t use = it / NBUF;
        if (!mbar_wait(&tempty[buf], (use & 1) ^ 1)) {
          s_abort = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dt = tbase + (uint32_t)buf * 256;
        for (int c = 0; c < nch; ++c, ++g) {
          const int st = g % CPL_NSTAGE;
          if (!mbar_wait(&full[st], (g / CPL_NSTAGE) & 1)) {
            s_abort = 1;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t soff = (uint64_t)((st * STAGE) >> 4);
          // A plane pp against B planes 0 .. 6 - pp stacked along N: levels
          // pp .. 6 in one instruction, or, above N = 256, two equal halves
          // (as in the trailing update)
#pragma unroll
          for (int pp = 0; pp < NSLICE; ++pp) {
            const int n = N * (NSLICE - pp);
            const int nh = n <= 256 ? n : n / 2;
#pragma unroll
            for (int off = 0; off < n; off += nh)
              mma_f16_desc(dt + (uint32_t)(pp * N + off), adesc0 + soff + (uint64_t)(pp * 4096 >> 4),
                           bdesc0 + soff + (uint64_t)((off * 16) >> 4),
                           (1u << 4) | ((uint32_t)(nh >> 3) << 17) | ((128u >> 4) << 24),
                           (c == 0 && pp == 0) ? 0u : 1u);
          }
          mma_commit(&empty[st]);
        }
        if (s_abort) break;
        mma_commit(&tfull[buf]);
      }
    }
  } else if (warp == CPL_RHS_WARP) {
    // ---------------- right-hand-side rows (FP64), problems round-robin ----------------
    for (int p = blockIdx.x; p < nprob; p += gridDim.x) {
      const Prob& P = probs[p];
      if (P.mode != 1 || s >= P.nt128 || P.status[1]) continue;
      const size_t ld = (size_t)P.ld;
      const int kb = s * NB + sq * QW;  // first source column; ns == NQ source quarters
      const int jb = s * NB + dq * QW;  // first destination column
      for (int b = 0; b < P.nrhs; ++b) {
        const double* zrow = P.K + P.Nc + b;  // right-hand-side row b: column c at c * ld
        double zr[NQ];                        // lane l: the row's entries at source columns l, l + 32
#pragma unroll
        for (int h = 0; h < NQ; ++h) zr[h] = zrow[(size_t)(kb + 32 * h + lane) * ld];
#pragma unroll
        for (int h = 0; h < NQ; ++h) {  // destination column jb + 32 h + lane
          const int j = jb + 32 * h + lane;
          double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
          for (int h2 = 0; h2 < NQ; ++h2)
#pragma unroll 8
            for (int k = 0; k < 32; ++k)
              acc[k & 3] = fma(__shfl_sync(0xffffffffu, zr[h2], k), P.K[(size_t)(kb + 32 * h2 + k) * ld + j], acc[k & 3]);
          P.K[(size_t)j * ld + P.Nc + b] -= (acc[0] + acc[1]) + (acc[2] + acc[3]);
        }
      }
    }
  } else {
    // ---------------- epilogue (warps 0-15): row = TMEM lane ----------------
    constexpr int NH = N / (CPL_EPI_WARPS / 4);  // columns per warp
    const int lq = warp & 3, hf = warp >> 2;
    uint32_t it = 0;
    for (uint32_t k = 0;; ++k, ++it) {
      int id;
      if (!next_tile(k, id)) {
        s_abort = 1;
        break;
      }
      if (id < 0) break;
      const int p = id >> 16, ti = id & 0xFFFF;
      const Prob& P = probs[p];
      const int buf = it % NBUF;
      const uint32_t use = it / NBUF;
      const int cd = s * NB + dq * QW;
      const int i = ti * NB + 32 * lq + lane;
      const bool live = i >= cd && i < P.Nc;
      const size_t ld = (size_t)P.ld;
      double* kcol = P.K + (size_t)(cd + hf * NH) * ld + i;
      // the first group's K entries, the row scale and this half's column
      // scales (lane l: column hf NH + l) load while the MMAs run
      double kv[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) kv[jj] = live ? kcol[(size_t)jj * ld] : 0.0;
      const int ei = P.escale[i < P.Nc ? i : 0] - 62;
      const int ecol = P.escale[cd + hf * NH + (lane % NH)];
      if (!mbar_wait(&tfull[buf], use & 1)) {
        s_abort = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
      for (int g = 0; g < NH / 8; ++g) {
        uint32_t v[NSLICE][8];
#pragma unroll
        for (int l = 0; l < NSLICE; ++l)
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                       : "=r"(v[l][0]), "=r"(v[l][1]), "=r"(v[l][2]), "=r"(v[l][3]), "=r"(v[l][4]),
                         "=r"(v[l][5]), "=r"(v[l][6]), "=r"(v[l][7])
                       : "r"(tbase + (uint32_t)buf * 256 + ((uint32_t)(lq * 32) << 16) +
                             (uint32_t)(l * N + hf * NH + g * 8)));
        double kn[8];  // the next group's K entries
        const bool more = live && g + 1 < NH / 8;
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) kn[jj] = more ? kcol[(size_t)((g + 1) * 8 + jj) * ld] : 0.0;
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        // the exact level sums from their magic-added bits (see level_bits)
        // when every sum of the warp's group lies in (-2^22, 2^22): always
        // for N = 32 (7 x 32 x 2^14 < 2^22); for N = 64 checked on the raw
        // sums, the warp converting with F2I otherwise -- so no second TMEM
        // read is needed and the buffer is released as soon as the tile's
        // last group is in registers, before that group converts
        bool slow = false;
        if constexpr (NQ > 1) {
          float mx = 0.0f;
#pragma unroll
          for (int l = 0; l < NSLICE; ++l)
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) mx = fmaxf(mx, fabsf(__uint_as_float(v[l][jj])));
          slow = !__all_sync(0xffffffffu, mx < 4194304.0f);
        }
        if (g == NH / 8 - 1) {
          asm volatile("tcgen05.fence::before_thread_sync;");
          mbar_arrive(&tempty[buf]);  // this buffer is free for the tile after next (or the next, N = 64)
        }
        if (!slow) {
#pragma unroll
          for (int l = 0; l < NSLICE; ++l)
#pragma unroll
            for (int jj = 0; jj < 8; ++jj) v[l][jj] = level_bits(v[l][jj]);
        }
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) {
          const int ej = __shfl_sync(0xffffffffu, ecol, g * 8 + jj);
          long long W;
          if (slow) {
            int S[NSLICE];
#pragma unroll
            for (int l = 0; l < NSLICE; ++l) S[l] = __float2int_rn(__uint_as_float(v[l][jj]));
            W = levels_to_w64(S);
          } else {
            W = level_bits_to_w64(v, jj);
          }
          // |sum_k L_ik L_jk| <= sqrt(K_ii K_jj) < 2^(e_i + e_j): |W| < 2^62
          kv[jj] -= w64_to_double(W, ei + ej);
        }
        if (live) {
#pragma unroll
          for (int jj = 0; jj < 8; ++jj) kcol[(size_t)(g * 8 + jj) * ld] = kv[jj];
        }
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) kv[jj] = kn[jj];
      }
      if (ti == s) {
        // the problem's own row tile holds quarter dq's diagonal block: factor it
        bar_sync_n(1, CPL_EPI);  // every coupled entry of the tile written and visible
        if (warp < 4 && !*(volatile int*)&P.status[1])
          potf2_block<QW>(P, cd, s * (NB / QW) + dq, tid, s_potf, 2);
      }
    }
  }
  __syncthreads();
  if (s_abort) {
    // a bounded wait gave up: the copies and MMAs this CTA issued finish
    // (bounded waits) before it frees its TMEM and exits
    if (warp == CPL_TMA_WARP && lane == 0) drain_ring(full, CPL_NSTAGE, issued);
    if (warp == CPL_MMA_WARP && lane == 0) drain_mmas(drain);
    __syncthreads();
    if (tid == 0)
      for (int k = 0; k < nprob; ++k) atomicExch(&probs[k].status[2], 1);
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == CPL_MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase));
}

// ---------------------------------------------------------------------------
// right-hand-side rows: C_qj -= sum_k Z_qk L_jk over the panel (FP64)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_border_update(const Prob* __restrict__ probs, int s) {
  const Prob& P = probs[blockIdx.y];
  if (P.mode != 1 || s + 1 >= P.nt128 || P.status[1]) return;
  __shared__ double Z[MAX_RHS][NB];
  const size_t ld = (size_t)P.ld;
  const int c0 = s * NB;
  for (int e = threadIdx.x; e < MAX_RHS * NB; e += blockDim.x) {
    const int q = e / NB, k = e % NB;
    Z[q][k] = q < P.nrhs ? P.K[(size_t)(c0 + k) * ld + P.Nc + q] : 0.0;
  }
  __syncthreads();
  const int j = c0 + NB + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= P.Nc) return;
  // one or two right-hand sides, chosen outside the loop (FP64 operations
  // for an absent second row would still cost the FP64 pipe)
  if (P.nrhs > 1) {
    double a0 = 0.0, a1 = 0.0;
    for (int k = 0; k < NB; ++k) {
      const double l = P.K[(size_t)(c0 + k) * ld + j];
      a0 = fma(Z[0][k], l, a0);
      a1 = fma(Z[1][k], l, a1);
    }
    P.K[(size_t)j * ld + P.Nc] -= a0;
    P.K[(size_t)j * ld + P.Nc + 1] -= a1;
  } else {
    double a0 = 0.0;
    for (int k = 0; k < NB; ++k) a0 = fma(Z[0][k], P.K[(size_t)(c0 + k) * ld + j], a0);
    P.K[(size_t)j * ld + P.Nc] -= a0;
  }
}

// ---------------------------------------------------------------------------
// quarter panel solve with a tensor-core coupling inside the quarter: row r of
// the panel below quarter q's diagonal block solves x L_qq^T = b by forward
// substitution in FP64, one thread per row, but in two halves of 16 columns:
// after the first half, its digit planes (the same 55-bit fixed point and 7
// fp16 digits as everywhere) go to shared memory together with those of L_qq's
// lower-left 16 x 16 block, 7 tcgen05.mma (M = 128, K = 16; B's planes stacked
// along N, N = 16 (7 - p) for A plane p) form the coupling sum_{k<16} x_k L_jk
// with the same 7 digit-product levels as the trailing update (each level an
// exact integer in f32), and each thread subtracts it, converted with one
// rounding, from its row before solving the second half.  That halves the FP64
// substitution work of the quarter.  The right-hand-side rows (no digit scale)
// take the coupling in FP64.  Each thread also writes its row's digit planes,
// which is everything the couplings and the trailing update read of this
// quarter: their rows all lie below the quarter's diagonal block.  128 rows
// per CTA; 112 TMEM columns.
// ---------------------------------------------------------------------------
constexpr int TQ_H = 16;                               // half a quarter
constexpr uint32_t TQ_A_BYTES = NSLICE * 2 * 128 * 16;  // 28 KB: first-half digits of the CTA's 128 rows
constexpr uint32_t TQ_B_BYTES = NSLICE * 2 * 16 * 16;   // 3.5 KB: digits of L_qq rows 16..31, columns 0..15
constexpr uint32_t TQ_SMEM = TQ_A_BYTES + TQ_B_BYTES + 64;

// The 7 fp16 digit planes of 8 entries (one k-group of a row), packed: the
// 55-bit fixed point F of an entry in its row scale has the balanced digits
// d_p in [-128, 127] (p = 1..6, base 256, lowest last) and d_0 = the rest.
// G = F + sum_{k<6} 128 256^k turns them into plain bytes: byte 6 - p of G
// is d_p + 128, and G >> 48 is d_0 (|d_0| <= 128 when |x| <= 2^e).  A byte
// u under the fp16 exponent bits 0x64 is the half 1024 + u, so one HSUB2 of
// 1152 per pair of entries yields the digits exactly, with no conversion
// instruction; two byte permutes place a pair's bytes under the 0x64 bytes.
// A top digit outside [-128, 128] breaks the row's scale bound and sets
// *bad.
__device__ __forceinline__ void digits8_packed(const double* x, int e, bool* bad, uint4 out[NSLICE]) {
  unsigned lo[8], hi[8];
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const long long G = to_fixed55(x[kk], e, bad) + 0x808080808080LL;
    lo[kk] = (unsigned)G;
    hi[kk] = (unsigned)(G >> 32);
    if ((unsigned)(((int)hi[kk] >> 16) + 128) > 256u) *bad = true;
  }
  const __half2 off = __halves2half2(__ushort_as_half(0x6480), __ushort_as_half(0x6480));  // 1152
#pragma unroll
  for (int p = 0; p < NSLICE; ++p) {
    unsigned w[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      unsigned bits;
      if (p == 0) {  // d_0 + 128 may be 256: arithmetic, not a byte
        const unsigned u0 = (unsigned)(((int)hi[2 * m] >> 16) + 128);
        const unsigned u1 = (unsigned)(((int)hi[2 * m + 1] >> 16) + 128);
        bits = (0x6400u + u0) | ((0x6400u + u1) << 16);
      } else {
        const int q = 6 - p;  // byte of G: byte q & 3 of the low or high word
        const unsigned wa = q < 4 ? lo[2 * m] : hi[2 * m], wb = q < 4 ? lo[2 * m + 1] : hi[2 * m + 1];
        const unsigned t = __byte_perm(wa, 0x64646464u, 0x4440u | (unsigned)(q & 3));  // [a_q, 64, 64, 64]
        bits = __byte_perm(wb, t, 0x7054u | ((unsigned)(q & 3) << 8));                  // [a_q, 64, b_q, 64]
      }
      const __half2 h = __hsub2(*reinterpret_cast<const __half2*>(&bits), off);
      w[m] = *reinterpret_cast<const unsigned*>(&h);
    }
    out[p] = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

__global__ void __launch_bounds__(128, 4) k_trsm_quarter(const Prob* __restrict__ probs, int col0_step, int col0_off) {
  const Prob& P = probs[blockIdx.y];
  const int col0 = col0_step + col0_off;
  const int last = P.nrt ? P.nrt - 1 : P.nsteps;  // last 64-row tile: factor rows, then the right-hand-side rows
  const int row_end = (last + 1) * TB;
  const int rbase = col0 + QW + blockIdx.x * 128;
  if (P.mode != 1 || col0 >= P.Nc || rbase >= row_end) return;
  __shared__ int s_skip;
  if (threadIdx.x == 0) s_skip = *(volatile int*)&P.status[1];  // one read: the exit below is block-uniform
  __syncthreads();
  if (s_skip) return;
  extern __shared__ __align__(1024) unsigned char smt[];
  unsigned char* As = smt;               // [plane][k-group 2][row 128][8 x fp16]
  unsigned char* Bs = smt + TQ_A_BYTES;  // [k-group 2][plane][row 16][8 x fp16]: planes stacked along N
  uint64_t* bar = reinterpret_cast<uint64_t*>(smt + TQ_A_BYTES + TQ_B_BYTES);
  __shared__ double L[QW * QW];  // L[c * QW + k] = L_ck
  __shared__ double rd[QW];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const size_t ld = (size_t)P.ld;
  const double* Ld = P.K + (size_t)col0 * ld + col0;
  for (int e = tid; e < QW * QW; e += 128) {
    const int c = e % QW, k = e / QW;  // coalesced over c
    L[c * QW + k] = Ld[(size_t)k * ld + c];
  }
  if (tid == 0) {
    s_fail = 0;
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(su32(&s_tmem)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = s_tmem;
  bool bad = false;
  if (tid < QW) rd[tid] = 1.0 / L[tid * QW + tid];
  if (tid >= 64 && tid < 96) {
    // B: rows 16..31 of L_qq, columns 0..15 (one thread per row and k-group)
    const int t = tid - 64, j = TQ_H + (t >> 1), g = t & 1;
    uint4 d[NSLICE];
    digits8_packed(&L[j * QW + g * 8], P.escale[col0 + j], &bad, d);
#pragma unroll
    for (int p = 0; p < NSLICE; ++p)
      *reinterpret_cast<uint4*>(Bs + g * (NSLICE * 256) + p * 256 + (j - TQ_H) * 16) = d[p];
  }
  __syncthreads();
  const int r = rbase + tid;
  const bool live = r < row_end;
  const bool fac = live && r < P.Nc;  // factor row: digit planes and the tensor-core coupling
  double x[QW];
  double* row = P.K + (size_t)col0 * ld + r;
#pragma unroll
  for (int c = 0; c < QW; ++c) x[c] = live ? row[(size_t)c * ld] : 0.0;
  // first half
#pragma unroll
  for (int c = 0; c < TQ_H; ++c) {
    double a = x[c];
#pragma unroll
    for (int k = 0; k < c; ++k) a = fma(-x[k], L[c * QW + k], a);
    x[c] = a * rd[c];
  }
  const int er = fac ? P.escale[r] : 0;
  unsigned char* gbase = P.slices + (size_t)(r / NB) * NSLICE * SLICE_BYTES + (size_t)(r % NB) * 16;
  const int kg0 = (col0 % NB) / 8;
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    uint4 d[NSLICE];
    if (fac) {
      digits8_packed(&x[g * 8], er, &bad, d);
    } else {
#pragma unroll
      for (int p = 0; p < NSLICE; ++p) d[p] = make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int p = 0; p < NSLICE; ++p) {
      const uint4 v = d[p];
      *reinterpret_cast<uint4*>(As + p * 4096 + g * 2048 + tid * 16) = v;
      if (fac) *reinterpret_cast<uint4*>(gbase + (size_t)p * SLICE_BYTES + (size_t)(kg0 + g) * 2048) = v;
    }
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // digits visible to the tensor cores
  __syncthreads();
  if (tid == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint64_t a0 = smem_desc(su32(As), 2048, 128), b0 = smem_desc(su32(Bs), NSLICE * 256, 128);
    // A plane pp against B planes 0 .. 6 - pp stacked along N: levels pp .. 6
#pragma unroll
    for (int pp = 0; pp < NSLICE; ++pp)
      mma_f16_desc(tmem + (uint32_t)pp * 16, a0 + (uint64_t)((pp * 4096) >> 4), b0,
                   (1u << 4) | ((uint32_t)(16 * (NSLICE - pp) >> 3) << 17) | ((128u >> 4) << 24), pp == 0 ? 0u : 1u);
    mma_commit(bar);
  }
  if (!mbar_wait(bar, 0)) s_fail = 1;
  asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    uint32_t v[NSLICE][8];
#pragma unroll
    for (int l = 0; l < NSLICE; ++l)
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                   : "=r"(v[l][0]), "=r"(v[l][1]), "=r"(v[l][2]), "=r"(v[l][3]), "=r"(v[l][4]), "=r"(v[l][5]),
                     "=r"(v[l][6]), "=r"(v[l][7])
                   : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(l * 16 + g * 8)));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (fac) {
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        int S[NSLICE];  // every level <= 7 x 16 x 128^2 < 2^22
#pragma unroll
        for (int l = 0; l < NSLICE; ++l) S[l] = small_f2i(__uint_as_float(v[l][jj]));
        const int j = TQ_H + g * 8 + jj;
        x[j] -= w64_to_double(levels_to_w64(S), er - 62 + P.escale[col0 + j]);
      }
    }
  }
  // right-hand-side rows: the coupling in FP64.  Only the warp holding a
  // problem's right-hand-side rows enters (a warp-uniform branch), so the
  // other warps do not issue these FP64 operations predicated off.
  if (__any_sync(0xffffffffu, live && !fac)) {
    if (live && !fac) {
#pragma unroll
      for (int j = TQ_H; j < QW; ++j) {
        double a = x[j];
#pragma unroll
        for (int k = 0; k < TQ_H; ++k) a = fma(-x[k], L[j * QW + k], a);
        x[j] = a;
      }
    }
  }
  // second half
#pragma unroll
  for (int c = TQ_H; c < QW; ++c) {
    double a = x[c];
#pragma unroll
    for (int k = TQ_H; k < c; ++k) a = fma(-x[k], L[c * QW + k], a);
    x[c] = a * rd[c];
  }
  if (fac) {
#pragma unroll
    for (int g = 2; g < 4; ++g) {
      uint4 d[NSLICE];
      digits8_packed(&x[g * 8], er, &bad, d);
#pragma unroll
      for (int p = 0; p < NSLICE; ++p)
        *reinterpret_cast<uint4*>(gbase + (size_t)p * SLICE_BYTES + (size_t)(kg0 + g) * 2048) = d[p];
    }
  }
  if (live) {
#pragma unroll
    for (int c = 0; c < QW; ++c) row[(size_t)c * ld] = x[c];
  }
  if (bad) atomicOr(&P.status[3], 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (tid == 0 && s_fail) {
    mbar_wait(bar, 0);  // the coupling MMAs complete (bounded) before TMEM is freed
    atomicExch(&P.status[2], 1);
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// host: TMA tensor maps over a problem's digit-plane buffer
// buffer layout: [row tile nt128][plane 7][k-group 16][row 128][8 fp16]; a (k-group, plane)
// block is 2 KB contiguous
// ---------------------------------------------------------------------------
int encode_slice_maps(void* host_maps, const void* slices, int nt128) {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!fn) {
      void* f = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
              cudaSuccess ||
          q != cudaDriverEntryPointSuccess || !f)
        return -1;
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    }
  }
  // A (k-group, plane) block of 128 rows x 16 B is 2 KB contiguous: describe it
  // as 4 rows of 256 fp16 (512 B) so each TMA request moves 512 B.
  const cuuint64_t dims[5] = {256, 4, 16, (cuuint64_t)NSLICE, (cuuint64_t)nt128};
  const cuuint64_t strides[4] = {512, 2048, (cuuint64_t)SLICE_BYTES, (cuuint64_t)NSLICE * SLICE_BYTES};
  const cuuint32_t boxA[5] = {256, 4, 2, NSLICE, 1};   // 128 rows
  const cuuint32_t boxB[5] = {256, 2, 2, NSLICE, 1};   // 64 rows
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUtensorMap* m = static_cast<CUtensorMap*>(host_maps);
  CUresult r = fn(&m[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, const_cast<void*>(slices), dims, strides, boxA, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return (int)r;
  r = fn(&m[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, const_cast<void*>(slices), dims, strides, boxB, es,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return (int)r;
  // boxes of 64 and 32 rows with the plane and k-group dimensions swapped:
  // they land as [k-group][plane][row], so the 7 planes of a k-group are one
  // operand of 7 x 64 (7 x 32) rows (the stacked-N MMAs of the trailing
  // update and the couplings)
  const cuuint64_t dimsS[5] = {256, 4, (cuuint64_t)NSLICE, 16, (cuuint64_t)nt128};
  const cuuint64_t stridesS[4] = {512, (cuuint64_t)SLICE_BYTES, 2048, (cuuint64_t)NSLICE * SLICE_BYTES};
  const cuuint32_t boxS[5] = {256, 2, NSLICE, 2, 1};
  const cuuint32_t boxS32[5] = {256, 1, NSLICE, 2, 1};
  r = fn(&m[2], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, const_cast<void*>(slices), dimsS, stridesS, boxS, es,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return (int)r;
  r = fn(&m[3], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, const_cast<void*>(slices), dimsS, stridesS, boxS32, es,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return (int)r;
}

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
static cudaError_t set_attrs() {
  cudaError_t e;
  if ((e = ensure_smem_attr((const void*)k_ozaki_update, SMEM_OZAKI_UPDATE, UPD_SMEM)) != cudaSuccess) return e;
  if ((e = ensure_smem_attr((const void*)k_couple<1>, SMEM_COUPLE1, CPL_SMEM)) != cudaSuccess) return e;
  return ensure_smem_attr((const void*)k_couple<2>, SMEM_COUPLE2, CPL_SMEM);
}

cudaError_t launch_scales(const Prob* probs, int nprob, int max_nc, cudaStream_t s) {
  k_scales<<<dim3((max_nc + 255) / 256, nprob), 256, 0, s>>>(probs);
  return cudaGetLastError();
}

cudaError_t launch_panel_prep(const Prob* probs, int nprob, int step, int max_nc, cudaStream_t s) {
  const int rows = max_nc - step * NB;
  if (step == 0 || rows <= 0) return cudaSuccess;
  k_panel_prep<<<dim3((rows + 255) / 256, NB / PP_COLS, nprob), 256, 0, s>>>(probs, step);
  return cudaGetLastError();
}

cudaError_t launch_trsm_quarter(const Prob* probs, int nprob, int step, int q, int max_rows, cudaStream_t s) {
  static_assert(TQ_SMEM + (QW * QW + QW) * sizeof(double) + 16 <= 48 * 1024, "no opt-in needed below 48 KB");
  const int rows = max_rows - (step * NB + q * QW + QW);
  if (rows <= 0) return cudaSuccess;
  k_trsm_quarter<<<dim3((rows + 127) / 128, nprob), 128, TQ_SMEM, s>>>(probs, step * NB, q * QW);
  return cudaGetLastError();
}

cudaError_t launch_couple(const Prob* probs, int nprob, int step, int sq, int ns, int dq, int nq,
                          const int* order, int total_tiles, int* counter, int num_sms, cudaStream_t s) {
  cudaError_t e = set_attrs();
  if (e != cudaSuccess) return e;
  int grid = total_tiles < num_sms ? total_tiles : num_sms;
  if (grid < 1) grid = 1;  // the right-hand-side rows still need their coupling
  if (nq == 1)
    k_couple<1><<<grid, CPL_THREADS, CPL_SMEM, s>>>(probs, nprob, step, sq, ns, dq, order, total_tiles, counter);
  else
    k_couple<2><<<grid, CPL_THREADS, CPL_SMEM, s>>>(probs, nprob, step, sq, ns, dq, order, total_tiles, counter);
  return cudaGetLastError();
}

cudaError_t launch_ozaki_update(const Prob* probs, int nprob, int step, int max_nt128,
                                const unsigned long long* tiles, int total_tiles, int num_sms, cudaStream_t s) {
  cudaError_t e = set_attrs();
  if (e != cudaSuccess) return e;
  if (max_nt128 - step - 1 <= 0 || total_tiles <= 0) return cudaSuccess;
  const int grid = total_tiles < num_sms ? total_tiles : num_sms;
  k_ozaki_update<<<grid, UPD_THREADS, UPD_SMEM, s>>>(probs, nprob, step, tiles, total_tiles);
  return cudaGetLastError();
}

cudaError_t launch_border_update(const Prob* probs, int nprob, int step, int max_nc, cudaStream_t s) {
  const int cols = max_nc - (step + 1) * NB;
  if (cols <= 0) return cudaSuccess;
  k_border_update<<<dim3((cols + 255) / 256, nprob), 256, 0, s>>>(probs, step);
  return cudaGetLastError();
}

}  // namespace fgpu
