// C-ABI of the engine: contexts (one training set each), a per-context pool of
// workers (stream + workspace + captured CUDA graph) for the plain
// one-particle-per-call path, and graph-captured batch plans.
#include "../../include/fgpu.h"
#include "fgpu_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <atomic>
#include <mutex>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

using namespace fgpu;

namespace {

thread_local std::string t_err;
thread_local long long t_launches = 0;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? FGPU_ENOMEM : FGPU_ECUDA, "%s: %s (%s:%d)", \
                  #call, cudaGetErrorString(e_), __FILE__, __LINE__);                     \
  } while (0)

int round_up(int v, int m) { return (v + m - 1) / m * m; }

// Compile the postfix spec into the device-side Spec and the plane list.
// Returns 0 or an error code (message set).
int compile_spec(const int* kspec, int nkspec, int d, Spec& sp, std::vector<int>& plane_dim,
                 std::vector<int>& plane_kind) {
  memset(&sp, 0, sizeof(sp));
  int depth = 0, i = 0, param = 0;
  while (i < nkspec) {
    const int op = kspec[i];
    if (op >= FGPU_RBF && op <= FGPU_CONSTANT) {
      if (i + 1 >= nkspec) return fail(FGPU_EINVAL, "kspec: truncated leaf at %d", i);
      const int n = kspec[i + 1];
      if (n < 0 || i + 2 + n > nkspec) return fail(FGPU_EINVAL, "kspec: bad leaf length at %d", i);
      if (op == FGPU_CONSTANT && n != 0) return fail(FGPU_EINVAL, "kspec: constant leaf takes no dims");
      if (op != FGPU_CONSTANT && n == 0) return fail(FGPU_EINVAL, "kspec: leaf with no active dims");
      if (sp.nleaf >= MAX_LEAF) return fail(FGPU_EINVAL, "kspec: more than %d leaves", MAX_LEAF);
      if (sp.npost >= MAX_POST) return fail(FGPU_EINVAL, "kspec: expression too long");
      Leaf& L = sp.leaf[sp.nleaf];
      L.type = op;
      L.n = n;
      L.plane0 = (int)plane_dim.size();
      L.param0 = param;
      if (op == FGPU_RBF_CYCLIC && n != d)
        return fail(FGPU_EINVAL,
                    "kspec: rbf-cyclic needs active dims = all %d features (the reference applies "
                    "its lengthscale to the whole cyclic distance tensor)", d);
      for (int k = 0; k < n; ++k) {
        const int dim = kspec[i + 2 + k];
        if (dim < 1 || dim > d) return fail(FGPU_EINVAL, "kspec: active dim %d outside 1..%d", dim, d);
        if (op == FGPU_PERIODIC) {
          plane_dim.push_back(dim - 1);
          plane_kind.push_back(1);  // sin(x/2)
          plane_dim.push_back(dim - 1);
          plane_kind.push_back(2);  // cos(x/2)
        } else if (op != FGPU_LINEAR) {
          plane_dim.push_back(dim - 1);
          plane_kind.push_back(op == FGPU_RBF_CYCLIC && (dim % 3) == 0 ? 3 : 0);
        }
      }
      param += (op == FGPU_CONSTANT) ? 1 : n;
      sp.post[sp.npost++] = (int8_t)sp.nleaf;
      sp.nleaf++;
      depth++;
      i += 2 + n;
    } else if (op == FGPU_SUM || op == FGPU_PROD) {
      if (depth < 2) return fail(FGPU_EINVAL, "kspec: operator at %d without two operands", i);
      if (sp.npost >= MAX_POST) return fail(FGPU_EINVAL, "kspec: expression too long");
      sp.post[sp.npost++] = (op == FGPU_SUM) ? P_SUM : P_PROD;
      depth--;
      i += 1;
    } else {
      return fail(FGPU_EINVAL, "kspec: bad opcode %d at %d", op, i);
    }
  }
  if (depth != 1) return fail(FGPU_EINVAL, "kspec: does not reduce to one kernel");
  if ((int)plane_dim.size() > MAX_PLANES)
    return fail(FGPU_EINVAL, "kspec: %d feature planes exceed the limit %d", (int)plane_dim.size(), MAX_PLANES);
  if (param > MAX_PARAMS - 1) return fail(FGPU_EINVAL, "kspec: %d parameters exceed the limit", param);
  sp.nplanes = (int)plane_dim.size();
  sp.nkparams = param;
  for (int p = 0; p < sp.nplanes; ++p) sp.cyclic[p] = plane_kind[p] == 3 ? 1 : 0;
  return 0;
}

// Tensor-core build eligibility (tensor-core mode): every leaf rbf, periodic,
// linear or constant; one or two rbf / periodic leaves whose feature columns,
// each rounded up to 16, fit the 128 digit columns of the panel buffer.  The
// process-wide build mode (fgpu_set_build_mode; FGPU_BUILD=fp64 at load)
// can keep the FP64 dot-product build instead.
// Atomic: contexts may be created from several host threads while another
// thread switches the mode.
std::atomic<int> g_build_mode{-1};  // 1: tensor-core build where eligible, 0: FP64 dot-product build
int build_mode() {
  int m = g_build_mode.load(std::memory_order_relaxed);
  if (m < 0) {
    const char* v = getenv("FGPU_BUILD");
    const int env = (v && (strcmp(v, "fp64") == 0 || strcmp(v, "0") == 0)) ? 0 : 1;
    g_build_mode.compare_exchange_strong(m, env, std::memory_order_relaxed);  // m: the value now set
    if (m < 0) m = env;
  }
  return m;
}

void plan_tc_build(Spec& sp) {
  sp.tc_build = 0;
  sp.ndot = 0;
  if (build_mode() == 0) return;
  int koff = 0;
  for (int l = 0; l < sp.nleaf; ++l) {
    const Leaf& L = sp.leaf[l];
    if (L.type == FGPU_RBF_CYCLIC) return;
    if (L.type != FGPU_RBF && L.type != FGPU_PERIODIC) continue;
    if (sp.ndot == 2) return;
    const int nf = L.type == FGPU_PERIODIC ? 2 * L.n : L.n;
    const int k16 = round_up(nf, 16);
    if (koff + k16 > NB) return;
    int lg = 0;
    while ((1 << lg) < nf) ++lg;  // ceil(log2 nf)
    sp.dot_leaf[sp.ndot] = l;
    sp.dot_koff[sp.ndot] = koff;
    sp.dot_kch[sp.ndot] = k16 / 16;
    sp.dot_u[sp.ndot] = 60 - lg;
    koff += k16;
    sp.ndot++;
  }
  sp.tc_build = sp.ndot > 0 ? 1 : 0;
}

// Per-step tile tables of the persistent tensor-core update: for step s,
// prefix[s * (nprob + 1) + p] = tiles of problems < p.
struct UpdSched {
  // trailing-update tiles of every step, packed (problem << 40 | row tile
  // << 20 | column tile), problem by problem, column tile major
  unsigned long long* tiles_dev = nullptr;
  std::vector<size_t> tile_off;  // first tile of each step
  std::vector<int> totals;       // tiles per step
  int num_sms = 0;
  unsigned long long* build_tiles_dev = nullptr;  // tiles of the tensor-core build, packed like `tiles_dev`
  int build_total = 0;
  std::vector<int> row_totals;      // per step: 128-row tiles ti >= step over all problems (couplings)
  int* cpl_order_dev = nullptr;     // per step: (problem << 16 | ti) of its row tiles, own row tile first
  std::vector<size_t> cpl_off;      // offset of each step's order
  int* cpl_counter_dev = nullptr;   // per step x 3 couplings: tile counters, zeroed per evaluation
  int ncounters = 0;
  // a second captured branch: the right-hand-side rows' trailing update runs
  // beside the next step's panel conversion and quarter-0 factor, joined
  // before that step's panel solve
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};

void free_sched_sync(UpdSched& u) {
  if (u.fork) cudaEventDestroy(u.fork);
  if (u.join) cudaEventDestroy(u.join);
  if (u.side) cudaStreamDestroy(u.side);
  u.fork = u.join = nullptr;
  u.side = nullptr;
}

// One problem's device buffers.  They are carved from one block (`base`,
// owned by a worker; a batch plan carves them from its shared arena instead
// and leaves `base` null); the TMA tensor maps live in their own 512 bytes
// because they must outlive the arena's reuse by later waves of a plan.
struct Workspace {
  void* base = nullptr;
  double* K = nullptr;
  double* logdet_part = nullptr;
  int* status = nullptr;
  double* out = nullptr;
  double* z = nullptr;
  // tensor-core mode
  int* escale = nullptr;
  double* pw2 = nullptr;
  long long* acc = nullptr;
  unsigned char* slices = nullptr;
  unsigned char* tmaps = nullptr;  // 4 x 128 B TMA tensor maps over slices (128-, 64-row boxes; 64, 32 rows, planes stacked)
  double* splanes = nullptr;       // theta-scaled planes (dot-product build)
  double* norms = nullptr;
  long long* fnorm = nullptr;      // tensor-core build: W_ii of the distance leaves
  double* fcoef = nullptr;         // tensor-core build: expression coefficients
  int* fscale = nullptr;           // tensor-core build: leaf scales
};

// Process-wide default trailing-update mode for contexts created from now on:
// 1 = tcgen05 split-integer update (128-wide panels), 0 = FP64 mma.sync.
// The environment variable FGPU_TRAILING=fp64 selects 0 at load time.
std::atomic<int> g_default_mode{-1};
int default_mode() {
  int m = g_default_mode.load(std::memory_order_relaxed);
  if (m < 0) {
    const char* v = getenv("FGPU_TRAILING");
    const int env = (v && (strcmp(v, "fp64") == 0 || strcmp(v, "0") == 0)) ? 0 : 1;
    g_default_mode.compare_exchange_strong(m, env, std::memory_order_relaxed);  // m: the value now set
    if (m < 0) m = env;
  }
  return m;
}

// Optional per-launch event pairs for stage timing (captured into the graph).
struct StageEvents {
  int only = -1;                // >= 0: time only the launches of this stage
  std::vector<int> stage;
  std::vector<cudaEvent_t> ev;  // 2 per launch
  void clear() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear();
    stage.clear();
  }
};


}  // namespace

struct Worker {
  cudaStream_t stream = nullptr;
  Workspace ws;
  double* theta_d = nullptr;
  Prob* prob_d = nullptr;
  double* h_stage = nullptr;  // pinned: theta | out(4) | status(4 ints as doubles)
  int* h_status = nullptr;
  cudaGraphExec_t graph = nullptr;
  long long graph_kernels = 0;
  bool busy = false;
  UpdSched sched;
};

// Adjoint workspace (FP64 geometry): K with the right-hand-side tile and N
// identity rows below it, K^-1, per-CTA partials.
struct GradWS {
  int Nc = 0, ld = 0, nsteps = 0, nrt = 0;
  Workspace ws;
  double* kinv = nullptr;
  double* gpart = nullptr;
  double* theta_d = nullptr;
  double* g_d = nullptr;
  Prob* prob_d = nullptr;
  cudaStream_t stream = nullptr;
  double* h_stage = nullptr;  // pinned: out(8) | g(ntheta) | status (as ints)
};

struct fgpu_ctx {
  int device = 0;
  int mode = 1;
  double* planes64_d = nullptr;  // FP64-mode planes (x; sin(x/2), cos(x/2)) for the adjoint
  GradWS* grad = nullptr;
  std::mutex grad_mu;
  int nt128 = 0;
  int N = 0, d = 0, Nc = 0, ld = 0, nsteps = 0, nrhs = 1, likelihood = 0, optimise_noise = 0;
  int nkparams = 0, ntheta = 0;
  double noise = 0.0;
  Spec spec{};
  Spec* spec_d = nullptr;
  double* planes_d = nullptr;
  double* plane_max_d = nullptr;  // nplanes: max_i |planes[p][i]| (tensor-core build scales)
  double* y_d = nullptr;
  double* mu_d = nullptr;
  std::mutex mu;
  std::vector<Worker*> workers;
};

// A batch plan.  Its problems run in waves (each wave one pass of the
// kernels over its problems; the waves one after the other in the same
// graph) whose workspaces share one arena: a batch whose workspaces do not
// fit the device memory budget at once still runs in one graph replay.
// probs_d holds the problems in wave order; order[k] is the caller's index
// of wave-order problem k (outputs land at the caller's index).
struct PlanWave {
  int first = 0, count = 0;  // range of probs_d
  int max_nsteps = 0, max_nplanes = 0;
  size_t bytes = 0;          // arena bytes this wave's workspaces span
  UpdSched sched;
};

struct fgpu_plan {
  int device = 0, nprob = 0, ldtheta = 0, mode = 0;
  std::vector<fgpu_ctx*> ctxs;
  std::vector<int> order;
  std::vector<PlanWave> waves;
  size_t arena_bytes = 0;
  std::vector<Prob> probs_h;
  Prob* probs_d = nullptr;
  double* theta_d = nullptr;
  double* ll_d = nullptr;
  int* info_d = nullptr;
  int* status_all = nullptr;
  std::vector<void*> allocations;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  long long graph_kernels = 0;
  double* h_theta = nullptr;
  double* h_ll = nullptr;
  int* h_info = nullptr;
  StageEvents* prof = nullptr;
  std::mutex mu;
};

namespace {

size_t K_elems(const fgpu_ctx* c) { return (size_t)c->ld * c->Nc; }

void fill_prob(Prob& p, const fgpu_ctx* c, const double* theta_d, const Workspace& ws) {
  memset(&p, 0, sizeof(p));
  p.N = c->N;
  p.Nc = c->Nc;
  p.ld = c->ld;
  p.nsteps = c->nsteps;
  p.nrhs = c->nrhs;
  p.likelihood = c->likelihood;
  p.optimise_noise = c->optimise_noise;
  p.nkparams = c->nkparams;
  p.noise = c->noise;
  p.planes = c->planes_d;
  p.y = c->y_d;
  p.mu = c->mu_d;
  p.spec = c->spec_d;
  p.theta = theta_d;
  p.K = ws.K;
  p.logdet_part = ws.logdet_part;
  p.status = ws.status;
  p.out = ws.out;
  p.z = ws.z;
  p.mode = c->mode;
  p.nt128 = c->nt128;
  p.escale = ws.escale;
  p.pw2 = ws.pw2;
  p.acc = ws.acc;
  p.slices = ws.slices;
  p.tmap_a = ws.tmaps;
  p.tmap_b = ws.tmaps ? ws.tmaps + 128 : nullptr;
  p.tmap_bs = ws.tmaps ? ws.tmaps + 256 : nullptr;
  p.tmap_bs32 = ws.tmaps ? ws.tmaps + 384 : nullptr;
  p.splanes = ws.splanes;
  p.norms = ws.norms;
  p.plane_max = c->plane_max_d;
  p.fnorm = ws.fnorm;
  p.fcoef = ws.fcoef;
  p.fscale = ws.fscale;
}

int build_sched(const std::vector<int>& nt128, const std::vector<int>& tc_build, UpdSched& u,
                std::vector<void*>* track) {
  const int nprob = (int)nt128.size();
  int ntmax = 0;
  for (int v : nt128) ntmax = std::max(ntmax, v);
  // step st, problem p: m = nt128 - st - 1 trailing row tiles; column-tile
  // pair q (tj = 2 (st + 1) + 2 q, + 1) holds row tiles st + 1 + q .. nt128 - 1
  std::vector<unsigned long long> tl;
  u.totals.assign(std::max(ntmax, 1), 0);
  u.tile_off.assign(std::max(ntmax, 1), 0);
  for (int st = 0; st < ntmax; ++st) {
    u.tile_off[st] = tl.size();
    for (int p = 0; p < nprob; ++p) {
      const int m = nt128[p] - st - 1;
      for (int q = 0; q < m; ++q)
        for (int half = 0; half < 2; ++half)
          for (int ti = st + 1 + q; ti < nt128[p]; ++ti)
            tl.push_back(((unsigned long long)p << 40) | ((unsigned long long)ti << 20) |
                         (unsigned long long)(2 * (st + 1) + 2 * q + half));
    }
    u.totals[st] = (int)(tl.size() - u.tile_off[st]);
  }
  if (tl.empty()) tl.push_back(0);
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&u.num_sms, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaStreamCreateWithFlags(&u.side, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&u.fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&u.join, cudaEventDisableTiming));
  CK(cudaMalloc(&u.tiles_dev, sizeof(unsigned long long) * tl.size()));
  if (track) track->push_back(u.tiles_dev);
  CK(cudaMemcpy(u.tiles_dev, tl.data(), sizeof(unsigned long long) * tl.size(), cudaMemcpyHostToDevice));
  // couplings: the row tiles ti >= step of every problem, in the order the
  // CTAs take them: every problem's own row tile (which also carries the
  // next quarter's diagonal factor) first
  {
    std::vector<int> ord;
    u.cpl_off.assign(std::max(ntmax, 1), 0);
    u.row_totals.assign(std::max(ntmax, 1), 0);
    for (int st = 0; st < ntmax; ++st) {
      u.cpl_off[st] = ord.size();
      for (int p = 0; p < nprob; ++p) u.row_totals[st] += std::max(0, nt128[p] - st);
      for (int p = 0; p < nprob; ++p)
        if (nt128[p] > st) ord.push_back((p << 16) | st);
      for (int p = 0; p < nprob; ++p)
        for (int ti = st + 1; ti < nt128[p]; ++ti) ord.push_back((p << 16) | ti);
    }
    if (ord.empty()) ord.push_back(0);
    CK(cudaMalloc(&u.cpl_order_dev, sizeof(int) * ord.size()));
    if (track) track->push_back(u.cpl_order_dev);
    CK(cudaMemcpy(u.cpl_order_dev, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice));
    u.ncounters = 3 * std::max(ntmax, 1);
    CK(cudaMalloc(&u.cpl_counter_dev, sizeof(int) * u.ncounters));
    if (track) track->push_back(u.cpl_counter_dev);
  }
  // tensor-core build: the whole lower triangle, nt128 (nt128 + 1) tiles of
  // 128 x 64 per eligible problem, column-tile pair major, row tile minor
  std::vector<unsigned long long> bl;
  for (int p = 0; p < nprob; ++p) {
    if (!tc_build[p]) continue;
    for (int q = 0; q < nt128[p]; ++q)
      for (int half = 0; half < 2; ++half)
        for (int ti = q; ti < nt128[p]; ++ti)
          bl.push_back(((unsigned long long)p << 40) | ((unsigned long long)ti << 20) |
                       (unsigned long long)(2 * q + half));
  }
  u.build_total = (int)bl.size();
  if (bl.empty()) bl.push_back(0);
  CK(cudaMalloc(&u.build_tiles_dev, sizeof(unsigned long long) * bl.size()));
  if (track) track->push_back(u.build_tiles_dev);
  CK(cudaMemcpy(u.build_tiles_dev, bl.data(), sizeof(unsigned long long) * bl.size(), cudaMemcpyHostToDevice));
  return 0;
}

int mark(StageEvents* pe, int stage, cudaStream_t s, bool begin) {
  if (!pe || (pe->only >= 0 && stage != pe->only)) return 0;
  cudaEvent_t e;
  CK(cudaEventCreate(&e));
  pe->ev.push_back(e);
  if (begin) pe->stage.push_back(stage);
  // External: becomes an event-record node of the captured graph
  CK(cudaEventRecordWithFlags(e, s, cudaEventRecordExternal));
  return 0;
}

#define STAGE(st, call)                        \
  do {                                         \
    int r_ = mark(pe, st, s, true);            \
    if (r_) return r_;                         \
    CK(call);                                  \
    r_ = mark(pe, st, s, false);               \
    if (r_) return r_;                         \
    ++n;                                       \
  } while (0)

// Enqueue the whole evaluation: reset, build, sweep, epilogue.
int enqueue_eval(const Prob* probs_d, int nprob, int max_nsteps, int max_nplanes, int* status_base,
                 size_t status_bytes, cudaStream_t s, long long* kernels, StageEvents* pe, int mode = 0,
                 const UpdSched* us = nullptr) {
  long long n = 0;
  CK(cudaMemsetAsync(status_base, 0, status_bytes, s));
  if (mode == 1) {
    // 128-wide panels; max_nsteps counts 64-column tiles
    const int nt = max_nsteps / 2, max_nc = max_nsteps * TB;
    CK(cudaMemsetAsync(us->cpl_counter_dev, 0, sizeof(int) * us->ncounters, s));
    STAGE(0, launch_prep_planes(probs_d, nprob, max_nc, s));
    if (us->build_total > 0) STAGE(0, launch_feat_digits(probs_d, nprob, nt, s));
    // FP64 dot-product build: every tile of the other problems, the
    // right-hand-side rows of all
    STAGE(0, launch_build_dot(probs_d, nprob, max_nsteps, max_nplanes, s));
    if (us->build_total > 0)
      STAGE(0, launch_build_tc(probs_d, nprob, us->build_tiles_dev, us->build_total, us->num_sms, s));
    STAGE(0, launch_scales(probs_d, nprob, max_nc, s));
    const int max_rows = max_nc + TB;  // the tallest problem's ld: factor rows + right-hand sides
    bool joins = false;                // a side branch awaits its join
    for (int step = 0; step < nt; ++step) {
      if (step > 0) STAGE(5, launch_panel_prep(probs_d, nprob, step, max_nc, s));
      // four 32-column quarters: FP64 diagonal factor, panel solve (which
      // writes the quarter's digit planes); tensor-core couplings quarter
      // 0 -> 1, half 0 -> 1, quarter 2 -> 3 before the quarter that needs
      // them, each of which also factors that quarter's diagonal block
      const int* order = us->cpl_order_dev + us->cpl_off[step];
      const int rows_total = us->row_totals[step];
      int* ctr = us->cpl_counter_dev + 3 * step;
      for (int q = 0; q < NB / QW; ++q) {
        if (q == 1) STAGE(8, launch_couple(probs_d, nprob, step, 0, 1, 1, 1, order, rows_total, ctr, us->num_sms, s));
        if (q == 2) STAGE(8, launch_couple(probs_d, nprob, step, 0, 2, 2, 2, order, rows_total, ctr + 1, us->num_sms, s));
        if (q == 3) STAGE(8, launch_couple(probs_d, nprob, step, 2, 1, 3, 1, order, rows_total, ctr + 2, us->num_sms, s));
        if (q == 0) STAGE(1, launch_potf2_quarter(probs_d, nprob, step, q, s));  // q > 0: inside the coupling
        if (q == 0 && joins) {  // the previous step's right-hand-side rows, before they are solved
          CK(cudaStreamWaitEvent(s, us->join, 0));
          joins = false;
        }
        STAGE(2, launch_trsm_quarter(probs_d, nprob, step, q, max_rows, s));  // also its digit planes
      }
      if (step + 1 < nt) {
        STAGE(3, launch_ozaki_update(probs_d, nprob, step, nt, us->tiles_dev + us->tile_off[step],
                                     us->totals[step], us->num_sms, s));
        // fork: the right-hand-side rows' FP64 update on the side branch,
        // beside the next step's panel conversion and quarter-0 factor
        CK(cudaEventRecord(us->fork, s));
        CK(cudaStreamWaitEvent(us->side, us->fork, 0));
        int r_ = mark(pe, 7, us->side, true);
        if (r_) return r_;
        CK(launch_border_update(probs_d, nprob, step, max_nc, us->side));
        r_ = mark(pe, 7, us->side, false);
        if (r_) return r_;
        ++n;
        CK(cudaEventRecord(us->join, us->side));
        joins = true;
      }
    }
    if (joins) CK(cudaStreamWaitEvent(s, us->join, 0));
    STAGE(4, launch_finalize(probs_d, nprob, s));
    if (kernels) *kernels = n;
    return 0;
  }
  STAGE(0, launch_build(probs_d, nprob, max_nsteps, max_nplanes, s));
  for (int step = 0; step < max_nsteps; ++step) {
    STAGE(1, launch_potf2(probs_d, nprob, step, s));
    STAGE(2, launch_trsm(probs_d, nprob, step, max_nsteps, s));
    if (max_nsteps - step - 1 > 0) STAGE(3, launch_update(probs_d, nprob, step, max_nsteps, s));
  }
  STAGE(4, launch_finalize(probs_d, nprob, s));
  if (kernels) *kernels = n;
  return 0;
}

int capture(cudaStream_t s, cudaGraphExec_t* exec, const Prob* probs_d, int nprob, int max_nsteps,
            int max_nplanes, int* status_base, size_t status_bytes, long long* kernels,
            StageEvents* pe = nullptr, int mode = 0, const UpdSched* us = nullptr) {
  if (mode == 1 && !us) return fail(FGPU_EINVAL, "internal: tensor-core mode without a tile schedule");
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_eval(probs_d, nprob, max_nsteps, max_nplanes, status_base, status_bytes, s, kernels, pe,
                        mode, us);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc != 0) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(FGPU_ECUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(FGPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
  return 0;
}

// Split a batch into waves whose workspaces fit `budget` bytes together.
// If the whole batch fits it is one wave in the caller's order; otherwise
// the problems are taken in decreasing workspace size and each wave is
// filled first-fit (a problem joins the current wave while it fits, else
// opens the next), so the largest problems share the first waves and the
// small ones pack densely into the last.  Returns FGPU_ENOMEM (message
// set) if a single problem exceeds the budget.
int plan_waves(const std::vector<size_t>& bytes, size_t budget, std::vector<std::vector<int>>& groups) {
  groups.clear();
  const int n = (int)bytes.size();
  size_t total = 0;
  for (size_t b : bytes) total += b;
  if (total <= budget) {
    groups.emplace_back();
    for (int i = 0; i < n; ++i) groups.back().push_back(i);
    return 0;
  }
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return bytes[a] > bytes[b]; });
  size_t cur = 0;
  for (int i : idx) {
    if (bytes[i] > budget)
      return fail(FGPU_ENOMEM, "problem %d needs %zu bytes of workspace; the device budget is %zu", i, bytes[i],
                  budget);
    if (groups.empty() || cur + bytes[i] > budget) {
      groups.emplace_back();
      cur = 0;
    }
    groups.back().push_back(i);
    cur += bytes[i];
  }
  return 0;
}

// Device memory a plan's workspaces may take at once: the environment
// variable FGPU_PLAN_MEM_BUDGET_MB if set, else the free memory less a
// reserve of max(1 GiB, 4 % of the device) for everything else.
size_t plan_memory_budget() {
  if (const char* v = getenv("FGPU_PLAN_MEM_BUDGET_MB")) {
    const double mb = atof(v);
    if (mb > 0) return (size_t)(mb * 1048576.0);
  }
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return (size_t)-1;  // unknown: one wave, and allocation reports the shortfall
  }
  const size_t reserve = std::max((size_t)1 << 30, tot / 25);
  return fr > reserve ? fr - reserve : 0;
}

// Capture a plan's waves, one after the other on the plan's stream, into
// one graph.
int capture_plan(fgpu_plan* p, cudaGraphExec_t* exec, long long* kernels, StageEvents* pe) {
  cudaStream_t s = p->stream;
  CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  long long total = 0;
  for (PlanWave& w : p->waves) {
    long long n = 0;
    rc = enqueue_eval(p->probs_d + w.first, w.count, w.max_nsteps, w.max_nplanes, p->status_all + 4 * w.first,
                      sizeof(int) * 4 * w.count, s, &n, pe, p->mode, p->mode == 1 ? &w.sched : nullptr);
    if (rc) break;
    total += n;
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (rc != 0) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(FGPU_ECUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(FGPU_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
  if (kernels) *kernels = total;
  return 0;
}

// Carve one problem's buffers from `base` (256-byte aligned pieces) and
// return the bytes they span; with base == nullptr only the size is
// computed.  The block needs no clearing: every buffer is written by the
// evaluation before it is read.
size_t layout_workspace(const fgpu_ctx* c, unsigned char* base, Workspace& ws) {
  size_t off = 0;
  auto take = [&](auto*& dst, size_t bytes) {
    off = (off + 255) / 256 * 256;
    dst = base ? reinterpret_cast<std::remove_reference_t<decltype(dst)>>(base + off) : nullptr;
    off += bytes;
  };
  const size_t nc = (size_t)c->Nc;
  take(ws.K, K_elems(c) * sizeof(double));
  // one log-det part per 64-column block (FP64 mode) or 32-column quarter (tensor-core mode)
  take(ws.logdet_part, sizeof(double) * 2 * (c->nsteps + 1));
  take(ws.out, sizeof(double) * 8);
  take(ws.z, sizeof(double) * nc);
  if (c->mode == 1) {
    take(ws.escale, sizeof(int) * nc);
    take(ws.pw2, sizeof(double) * nc);
    take(ws.acc, sizeof(long long) * acc_tiles(c->nt128) * ACC_TILE_ELEMS);
    take(ws.slices, (size_t)c->nt128 * NSLICE * SLICE_BYTES);
    take(ws.splanes, sizeof(double) * (size_t)std::max(c->spec.nplanes, 1) * nc);
    take(ws.norms, sizeof(double) * (size_t)MAX_LEAF * nc);
    take(ws.fnorm, sizeof(long long) * 2 * nc);
    take(ws.fcoef, sizeof(double) * 4);
    take(ws.fscale, sizeof(int) * 2);
  }
  return (off + 255) / 256 * 256;
}

size_t workspace_bytes(const fgpu_ctx* c) {
  Workspace tmp;
  return layout_workspace(c, nullptr, tmp);
}

// Encode the problem's four TMA tensor maps over ws.slices into the 512
// device bytes at `dst` (tensor-core mode only).
int write_tmaps(const fgpu_ctx* c, const Workspace& ws, unsigned char* dst) {
  if (c->mode != 1) return 0;
  alignas(64) unsigned char maps[512];
  const int er = encode_slice_maps(maps, ws.slices, c->nt128);
  if (er != 0) return fail(FGPU_ECUDA, "cuTensorMapEncodeTiled failed (%d)", er);
  CK(cudaMemcpy(dst, maps, 512, cudaMemcpyHostToDevice));
  return 0;
}

// A worker's own workspace: one block plus its tensor maps.  On failure
// nothing stays allocated and ws is left empty.
int alloc_workspace(const fgpu_ctx* c, Workspace& ws) {
  const size_t bytes = workspace_bytes(c);
  void* base = nullptr;
  cudaError_t e = cudaMalloc(&base, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();  // an allocation failure is not sticky; clear it
    return fail(e == cudaErrorMemoryAllocation ? FGPU_ENOMEM : FGPU_ECUDA,
                "workspace allocation of %zu bytes (N=%d): %s", bytes, c->N, cudaGetErrorString(e));
  }
  layout_workspace(c, static_cast<unsigned char*>(base), ws);
  ws.base = base;
  if (c->mode == 1) {
    e = cudaMalloc(&ws.tmaps, 512);
    int rc = e == cudaSuccess ? write_tmaps(c, ws, ws.tmaps)
                              : fail(FGPU_ENOMEM, "tensor-map allocation: %s", cudaGetErrorString(e));
    if (rc) {
      cudaFree(ws.tmaps);
      cudaFree(base);
      ws = Workspace{};
      return rc;
    }
  }
  return 0;
}

void free_worker(Worker* w) {
  if (!w) return;
  if (w->graph) cudaGraphExecDestroy(w->graph);
  cudaFree(w->ws.base);
  cudaFree(w->ws.status);
  cudaFree(w->ws.tmaps);
  cudaFree(w->theta_d);
  cudaFree(w->prob_d);
  cudaFree(w->sched.tiles_dev);
  cudaFree(w->sched.build_tiles_dev);
  cudaFree(w->sched.cpl_order_dev);
  cudaFree(w->sched.cpl_counter_dev);
  free_sched_sync(w->sched);
  if (w->h_stage) cudaFreeHost(w->h_stage);
  if (w->stream) cudaStreamDestroy(w->stream);
  delete w;
}

int make_worker(fgpu_ctx* c, Worker** out) {
  Worker* w = new (std::nothrow) Worker();
  if (!w) return fail(FGPU_ENOMEM, "worker allocation");
  int rc = 0;
  auto bail = [&](int r) {
    free_worker(w);
    return r;
  };
  if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(FGPU_ECUDA, "stream create failed"));
  if ((rc = alloc_workspace(c, w->ws)) != 0) return bail(rc);
  if (cudaMalloc(&w->ws.status, sizeof(int) * 4) != cudaSuccess) return bail(fail(FGPU_ENOMEM, "status alloc"));
  if (cudaMalloc(&w->theta_d, sizeof(double) * (c->ntheta + 1)) != cudaSuccess)
    return bail(fail(FGPU_ENOMEM, "theta alloc"));
  if (cudaMalloc(&w->prob_d, sizeof(Prob)) != cudaSuccess) return bail(fail(FGPU_ENOMEM, "desc alloc"));
  if (cudaMallocHost(&w->h_stage, sizeof(double) * (c->ntheta + 16)) != cudaSuccess)
    return bail(fail(FGPU_ENOMEM, "pinned alloc"));
  w->h_status = reinterpret_cast<int*>(w->h_stage + c->ntheta + 8);
  Prob p;
  fill_prob(p, c, w->theta_d, w->ws);
  if (cudaMemcpy(w->prob_d, &p, sizeof(Prob), cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(FGPU_ECUDA, "desc copy"));
  if (c->mode == 1 &&
      (rc = build_sched(std::vector<int>{c->nt128}, std::vector<int>{c->spec.tc_build}, w->sched, nullptr)) != 0)
    return bail(rc);
  if ((rc = capture(w->stream, &w->graph, w->prob_d, 1, c->nsteps, c->spec.nplanes, w->ws.status,
                    sizeof(int) * 4, &w->graph_kernels, nullptr, c->mode, &w->sched)) != 0)
    return bail(rc);
  *out = w;
  return 0;
}

Worker* acquire(fgpu_ctx* c, int* rc) {
  {
    std::lock_guard<std::mutex> lk(c->mu);
    for (Worker* w : c->workers)
      if (!w->busy) {
        w->busy = true;
        return w;
      }
  }
  Worker* w = nullptr;
  *rc = make_worker(c, &w);
  if (*rc) return nullptr;
  std::lock_guard<std::mutex> lk(c->mu);
  w->busy = true;
  c->workers.push_back(w);
  return w;
}

void release(fgpu_ctx* c, Worker* w) {
  std::lock_guard<std::mutex> lk(c->mu);
  w->busy = false;
}

// Plans that fgpu_loglik_batch built, keyed by the context list, least
// recently used first out: at most FGPU_PLAN_CACHE (default 8) are kept.
// Entries are shared, so an evicted plan is destroyed only after the last
// call still running it returns.
struct CachedPlan {
  std::shared_ptr<fgpu_plan> plan;
  unsigned long long used = 0;
};
std::mutex g_plan_mu;
std::map<std::vector<fgpu_ctx*>, CachedPlan> g_plans;
unsigned long long g_plan_clock = 0;

size_t plan_cache_limit() {
  const char* v = getenv("FGPU_PLAN_CACHE");
  const int n = v ? atoi(v) : 8;
  return (size_t)(n > 0 ? n : 1);
}

// Frees an adjoint workspace, complete or partly built (unset members are null).
void free_grad_ws(GradWS* g) {
  if (!g) return;
  for (void* q : {(void*)g->ws.K, (void*)g->ws.logdet_part, (void*)g->ws.status, (void*)g->ws.out,
                  (void*)g->ws.z, (void*)g->kinv, (void*)g->gpart, (void*)g->theta_d, (void*)g->g_d,
                  (void*)g->prob_d})
    cudaFree(q);
  if (g->h_stage) cudaFreeHost(g->h_stage);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}
struct GradWSDeleter {
  void operator()(GradWS* g) const { free_grad_ws(g); }
};
// A context that fgpu_create could not finish is destroyed with everything
// it had allocated.
struct CtxDeleter {
  void operator()(fgpu_ctx* c) const { fgpu_destroy(c); }
};

}  // namespace

extern "C" {

const char* fgpu_last_error(void) { return t_err.c_str(); }
const char* fgpu_version(void) { return "fgpu 0.1 sm_103a fp64"; }
long long fgpu_last_launch_count(void) { return t_launches; }

int fgpu_create(fgpu_ctx** out, int N, int d, const double* X, const double* y, const double* mu,
                const int* kspec, int nkspec, int likelihood, double noise, int optimise_noise) {
  t_err.clear();
  if (!out) return fail(FGPU_EINVAL, "ctx pointer is NULL");
  *out = nullptr;
  if (N < 1 || d < 1) return fail(FGPU_EINVAL, "N=%d d=%d must be positive", N, d);
  if (!X || !y || !kspec || nkspec < 1) return fail(FGPU_EINVAL, "NULL input array");
  if (likelihood != FGPU_MARGINAL && likelihood != FGPU_CONCENTRATED)
    return fail(FGPU_EINVAL, "likelihood %d is neither marginal (0) nor concentrated (1)", likelihood);
  if (likelihood == FGPU_MARGINAL && !mu) return fail(FGPU_EINVAL, "marginal likelihood needs mu");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(FGPU_ENODEV, "no CUDA device");
  std::unique_ptr<fgpu_ctx, CtxDeleter> c(new (std::nothrow) fgpu_ctx());
  if (!c) return fail(FGPU_ENOMEM, "context allocation");
  CK(cudaGetDevice(&c->device));
  std::vector<int> plane_dim, plane_kind;
  int rc = compile_spec(kspec, nkspec, d, c->spec, plane_dim, plane_kind);
  if (rc) return rc;
  c->N = N;
  c->d = d;
  c->mode = default_mode();
  if (c->mode == 1) plan_tc_build(c->spec);
  c->Nc = round_up(N, c->mode == 1 ? NB : TB);
  c->nt128 = c->Nc / NB;
  c->ld = c->Nc + TB;
  c->nsteps = c->Nc / TB;
  c->likelihood = likelihood;
  c->nrhs = likelihood == FGPU_CONCENTRATED ? 2 : 1;
  c->noise = noise;
  c->optimise_noise = optimise_noise ? 1 : 0;
  c->nkparams = c->spec.nkparams;
  c->ntheta = c->nkparams + c->optimise_noise;
  // feature planes, plane-major, padded to Nc.  FP64 mode: x, or the
  // half-angle pair sin(x/2), cos(x/2) for periodic dims.  Tensor-core mode
  // (dot-product build): rbf dims centred on their mean, periodic dims as
  // the pair cos(x), sin(x), rbf-cyclic dims raw.
  const int np = c->spec.nplanes;
  std::vector<double> planes((size_t)std::max(np, 1) * c->Nc, 0.0);
  std::vector<int> plane_leaf(np, 0);
  for (int l = 0; l < c->spec.nleaf; ++l) {
    const Leaf& L = c->spec.leaf[l];
    const int cnt = L.type == FGPU_PERIODIC ? 2 * L.n : (L.type == FGPU_LINEAR || L.type == FGPU_CONSTANT ? 0 : L.n);
    for (int q = 0; q < cnt; ++q) plane_leaf[L.plane0 + q] = L.type;
  }
  for (int p = 0; p < np; ++p) {
    const double* col = X + (size_t)plane_dim[p] * N;  // X(:, dim), column-major
    double* dst = planes.data() + (size_t)p * c->Nc;
    if (c->mode == 1 && plane_leaf[p] == FGPU_RBF) {
      double mean = 0.0;
      for (int i = 0; i < N; ++i) mean += col[i];
      mean /= N;
      for (int i = 0; i < N; ++i) dst[i] = col[i] - mean;
      continue;
    }
    for (int i = 0; i < N; ++i) {
      const double x = col[i];
      if (c->mode == 1 && plane_kind[p] == 1)
        dst[i] = std::cos(x);
      else if (c->mode == 1 && plane_kind[p] == 2)
        dst[i] = std::sin(x);
      else if (plane_kind[p] == 1)
        dst[i] = std::sin(x / 2.0);
      else if (plane_kind[p] == 2)
        dst[i] = std::cos(x / 2.0);
      else
        dst[i] = x;
    }
  }
  std::vector<double> yv(c->Nc, 0.0), mv(c->Nc, 0.0);
  for (int i = 0; i < N; ++i) {
    yv[i] = y[i];
    mv[i] = mu ? mu[i] : 0.0;
  }
  CK(cudaMalloc(&c->planes_d, planes.size() * sizeof(double)));
  CK(cudaMemcpy(c->planes_d, planes.data(), planes.size() * sizeof(double), cudaMemcpyHostToDevice));
  {
    std::vector<double> pmax(std::max(np, 1), 0.0);
    for (int p = 0; p < np; ++p)
      for (int i = 0; i < N; ++i) pmax[p] = std::max(pmax[p], std::fabs(planes[(size_t)p * c->Nc + i]));
    CK(cudaMalloc(&c->plane_max_d, pmax.size() * sizeof(double)));
    CK(cudaMemcpy(c->plane_max_d, pmax.data(), pmax.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  // FP64-mode planes for the adjoint (64-padded), whatever the context's mode
  {
    const int nc64 = round_up(N, TB);
    std::vector<double> p64((size_t)std::max(np, 1) * nc64, 0.0);
    for (int p = 0; p < np; ++p) {
      const double* col = X + (size_t)plane_dim[p] * N;
      double* dst = p64.data() + (size_t)p * nc64;
      for (int i = 0; i < N; ++i) {
        const double x = col[i];
        dst[i] = plane_kind[p] == 1 ? std::sin(x / 2.0) : (plane_kind[p] == 2 ? std::cos(x / 2.0) : x);
      }
    }
    CK(cudaMalloc(&c->planes64_d, p64.size() * sizeof(double)));
    CK(cudaMemcpy(c->planes64_d, p64.data(), p64.size() * sizeof(double), cudaMemcpyHostToDevice));
  }
  CK(cudaMalloc(&c->y_d, c->Nc * sizeof(double)));
  CK(cudaMemcpy(c->y_d, yv.data(), c->Nc * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&c->mu_d, c->Nc * sizeof(double)));
  CK(cudaMemcpy(c->mu_d, mv.data(), c->Nc * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&c->spec_d, sizeof(Spec)));
  CK(cudaMemcpy(c->spec_d, &c->spec, sizeof(Spec), cudaMemcpyHostToDevice));
  *out = c.release();
  return 0;
}

int fgpu_nparams(const fgpu_ctx* ctx) { return ctx ? ctx->ntheta : FGPU_EINVAL; }

int fgpu_set_build_mode(int mode) {
  const int prev = build_mode();
  if (mode != 0 && mode != 1) return fail(FGPU_EINVAL, "build mode must be 0 (fp64) or 1 (tensor cores)");
  g_build_mode.store(mode, std::memory_order_relaxed);
  return prev;
}

int fgpu_set_trailing_update(int mode) {
  const int prev = default_mode();
  if (mode != 0 && mode != 1) return fail(FGPU_EINVAL, "trailing-update mode must be 0 (fp64) or 1 (tcgen05)");
  g_default_mode.store(mode, std::memory_order_relaxed);
  return prev;
}

void fgpu_destroy(fgpu_ctx* ctx) {
  if (!ctx) return;
  {
    std::vector<std::shared_ptr<fgpu_plan>> drop;  // destroyed outside the lock
    std::lock_guard<std::mutex> lk(g_plan_mu);
    for (auto it = g_plans.begin(); it != g_plans.end();) {
      bool uses = false;
      for (fgpu_ctx* c : it->first) uses |= (c == ctx);
      if (uses) {
        drop.push_back(std::move(it->second.plan));
        it = g_plans.erase(it);
      } else {
        ++it;
      }
    }
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(ctx->device);
  for (Worker* w : ctx->workers) free_worker(w);
  free_grad_ws(ctx->grad);
  cudaFree(ctx->planes64_d);
  cudaFree(ctx->planes_d);
  cudaFree(ctx->plane_max_d);
  cudaFree(ctx->y_d);
  cudaFree(ctx->mu_d);
  cudaFree(ctx->spec_d);
  cudaSetDevice(prev);
  delete ctx;
}

int fgpu_loglik(fgpu_ctx* ctx, const double* theta, int ntheta, double* ll, int* info, double* alpha) {
  t_err.clear();
  t_launches = 0;
  if (!ctx || !theta || !ll || !info) return fail(FGPU_EINVAL, "NULL argument");
  if (ntheta != ctx->ntheta) return fail(FGPU_EINVAL, "ntheta=%d, context expects %d", ntheta, ctx->ntheta);
  for (int k = 0; k < ntheta; ++k)
    if (!std::isfinite(theta[k])) return fail(FGPU_EINVAL, "theta[%d] is not finite", k);
  CK(cudaSetDevice(ctx->device));
  int rc = 0;
  Worker* w = acquire(ctx, &rc);
  if (!w) return rc;
  struct Rel {
    fgpu_ctx* c;
    Worker* w;
    ~Rel() { release(c, w); }
  } rel{ctx, w};
  memcpy(w->h_stage, theta, sizeof(double) * ntheta);
  CK(cudaMemcpyAsync(w->theta_d, w->h_stage, sizeof(double) * ntheta, cudaMemcpyHostToDevice, w->stream));
  CK(cudaGraphLaunch(w->graph, w->stream));
  t_launches = w->graph_kernels;
  if (alpha) {
    CK(launch_backsolve(w->prob_d, 1, ctx->nsteps, nullptr, w->stream, &t_launches));
  }
  double* h_out = w->h_stage + ctx->ntheta;
  CK(cudaMemcpyAsync(h_out, w->ws.out, sizeof(double) * 4, cudaMemcpyDeviceToHost, w->stream));
  CK(cudaMemcpyAsync(w->h_status, w->ws.status, sizeof(int) * 4, cudaMemcpyDeviceToHost, w->stream));
  if (alpha) CK(cudaMemcpyAsync(alpha, w->ws.z, sizeof(double) * ctx->N, cudaMemcpyDeviceToHost, w->stream));
  CK(cudaStreamSynchronize(w->stream));
  if (w->h_status[2]) return fail(FGPU_ETIMEOUT, "a bounded wait in a kernel gave up (copy or MMA)");
  if (w->h_status[3] && !w->h_status[1])
    return fail(FGPU_ECUDA, "panel value outside its row scale bound (split-integer update)");
  *info = w->h_status[0];
  *ll = (*info == 0) ? h_out[0] : std::nan("");
  return 0;
}

namespace {
int make_grad_ws(fgpu_ctx* c, GradWS** out) {
  std::unique_ptr<GradWS, GradWSDeleter> g(new (std::nothrow) GradWS());  // freed whole on failure
  if (!g) return fail(FGPU_ENOMEM, "adjoint workspace");
  g->Nc = round_up(c->N, TB);
  g->nsteps = g->Nc / TB;
  g->ld = 2 * g->Nc + TB;
  g->nrt = g->ld / TB;
  const size_t nc = (size_t)g->Nc;
  CK(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  CK(cudaMalloc(&g->ws.K, sizeof(double) * (size_t)g->ld * nc));
  CK(cudaMalloc(&g->ws.logdet_part, sizeof(double) * (g->nsteps + 1)));
  CK(cudaMalloc(&g->ws.status, sizeof(int) * 4));
  CK(cudaMalloc(&g->ws.out, sizeof(double) * 8));
  CK(cudaMalloc(&g->ws.z, sizeof(double) * nc));
  CK(cudaMalloc(&g->kinv, sizeof(double) * nc * nc));
  CK(cudaMalloc(&g->gpart, sizeof(double) * (size_t)g->nsteps * g->nsteps * GRAD_SLOTS));
  CK(cudaMalloc(&g->theta_d, sizeof(double) * (c->ntheta + 1)));
  CK(cudaMalloc(&g->g_d, sizeof(double) * (c->ntheta + 1)));
  CK(cudaMalloc(&g->prob_d, sizeof(Prob)));
  CK(cudaMallocHost(&g->h_stage, sizeof(double) * (c->ntheta + 16)));
  Prob p;
  memset(&p, 0, sizeof(p));
  p.N = c->N;
  p.Nc = g->Nc;
  p.ld = g->ld;
  p.nsteps = g->nsteps;
  p.nrt = g->nrt;
  p.border_only = c->mode == 1 ? 1 : 0;
  p.nrhs = c->nrhs;
  p.likelihood = c->likelihood;
  p.optimise_noise = c->optimise_noise;
  p.nkparams = c->nkparams;
  p.noise = c->noise;
  p.planes = c->planes64_d;
  p.y = c->y_d;
  p.mu = c->mu_d;
  p.spec = c->spec_d;
  p.theta = g->theta_d;
  p.K = g->ws.K;
  p.logdet_part = g->ws.logdet_part;
  p.status = g->ws.status;
  p.out = g->ws.out;
  p.z = g->ws.z;
  p.mode = 0;
  p.kinv = g->kinv;
  p.gpart = g->gpart;
  CK(cudaMemcpy(g->prob_d, &p, sizeof(Prob), cudaMemcpyHostToDevice));
  *out = g.release();
  return 0;
}
}  // namespace

int fgpu_grad(fgpu_ctx* ctx, const double* theta, int ntheta, double* ll, double* dll, int* info) {
  t_err.clear();
  t_launches = 0;
  if (!ctx || !theta || !ll || !dll || !info) return fail(FGPU_EINVAL, "NULL argument");
  if (ntheta != ctx->ntheta) return fail(FGPU_EINVAL, "ntheta=%d, context expects %d", ntheta, ctx->ntheta);
  for (int k = 0; k < ntheta; ++k)
    if (!std::isfinite(theta[k])) return fail(FGPU_EINVAL, "theta[%d] is not finite", k);
  CK(cudaSetDevice(ctx->device));
  std::lock_guard<std::mutex> lk(ctx->grad_mu);
  if (!ctx->grad) {
    GradWS* g = nullptr;
    int rc = make_grad_ws(ctx, &g);
    if (rc) return rc;
    ctx->grad = g;
  }
  GradWS* g = ctx->grad;
  long long n = 0;
  Worker* w = nullptr;
  struct Rel {
    fgpu_ctx* c;
    Worker* w;
    ~Rel() {
      if (w) release(c, w);
    }
  } rel{ctx, nullptr};
  cudaStream_t s = g->stream;
  if (ctx->mode == 1) {
    // Tensor-core context: the evaluation itself (factor, log-likelihood,
    // alpha) is the plain path's graph; its factor L, alpha, the likelihood
    // epilogue's scalars and status are copied into the adjoint workspace,
    // whose FP64 sweep then only turns the identity rows into L^-T.  Every
    // step runs on the worker's stream; the worker is released after the
    // final synchronisation.
    int rc = 0;
    w = acquire(ctx, &rc);
    if (!w) return rc;
    rel.w = w;
    s = w->stream;
    memcpy(w->h_stage, theta, sizeof(double) * ntheta);
    CK(cudaMemcpyAsync(w->theta_d, w->h_stage, sizeof(double) * ntheta, cudaMemcpyHostToDevice, s));
    CK(cudaGraphLaunch(w->graph, s));
    n += w->graph_kernels;
    CK(launch_backsolve(w->prob_d, 1, ctx->nsteps, nullptr, s, &n));
    CK(cudaMemcpy2DAsync(g->ws.K, sizeof(double) * g->ld, w->ws.K, sizeof(double) * ctx->ld,
                         sizeof(double) * g->Nc, g->Nc, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->ws.z, w->ws.z, sizeof(double) * g->Nc, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->ws.out, w->ws.out, sizeof(double) * 8, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->ws.status, w->ws.status, sizeof(int) * 4, cudaMemcpyDeviceToDevice, s));
  }
  memcpy(g->h_stage, theta, sizeof(double) * ntheta);
  CK(cudaMemcpyAsync(g->theta_d, g->h_stage, sizeof(double) * ntheta, cudaMemcpyHostToDevice, s));
  if (ctx->mode != 1) {
    CK(cudaMemsetAsync(g->ws.status, 0, sizeof(int) * 4, s));
    CK(launch_build(g->prob_d, 1, g->nsteps, ctx->spec.nplanes, s));
    ++n;
  }
  CK(launch_identity_border(g->prob_d, g->Nc, s));
  ++n;
  for (int step = 0; step < g->nsteps; ++step) {
    if (ctx->mode != 1) {
      CK(launch_potf2(g->prob_d, 1, step, s));
      ++n;
    }
    CK(launch_trsm(g->prob_d, 1, step, g->nsteps, s, g->nrt));
    CK(launch_update(g->prob_d, 1, step, g->nsteps, s, g->nrt));
    n += 2;
  }
  if (ctx->mode != 1) {
    CK(launch_finalize(g->prob_d, 1, s));
    ++n;
    CK(launch_backsolve(g->prob_d, 1, g->nsteps, nullptr, s, &n));
  }
  CK(launch_syrk_inv(g->prob_d, g->nsteps, s));
  ++n;
  CK(enqueue_grad_passes(g->prob_d, g->nsteps, ctx->nkparams, ctx->optimise_noise, g->g_d, s, &n));
  double* h_out = g->h_stage;
  double* h_g = g->h_stage + 8;
  int* h_status = reinterpret_cast<int*>(g->h_stage + 8 + ctx->ntheta + 1);
  CK(cudaMemcpyAsync(h_out, g->ws.out, sizeof(double) * 8, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h_g, g->g_d, sizeof(double) * ntheta, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h_status, g->ws.status, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  t_launches = n;
  if (h_status[2]) return fail(FGPU_ETIMEOUT, "a bounded wait in a kernel gave up");
  if (h_status[3] && !h_status[1])
    return fail(FGPU_ECUDA, "panel value outside its row scale bound (split-integer update)");
  *info = h_status[0];
  *ll = (*info == 0) ? h_out[0] : std::nan("");
  for (int k = 0; k < ntheta; ++k) dll[k] = (*info == 0) ? h_g[k] : std::nan("");
  return 0;
}

int fgpu_plan_create(fgpu_plan** out, fgpu_ctx* const* ctxs, int nprob, int ldtheta) {
  t_err.clear();
  if (!out || !ctxs || nprob < 1) return fail(FGPU_EINVAL, "bad plan arguments");
  if (nprob > 65535) return fail(FGPU_EINVAL, "a plan holds at most 65535 problems (%d given)", nprob);
  *out = nullptr;
  std::unique_ptr<fgpu_plan> p(new (std::nothrow) fgpu_plan());
  if (!p) return fail(FGPU_ENOMEM, "plan allocation");
  p->nprob = nprob;
  p->device = ctxs[0] ? ctxs[0]->device : 0;
  int maxth = 0;
  for (int i = 0; i < nprob; ++i) {
    if (!ctxs[i]) return fail(FGPU_EINVAL, "ctxs[%d] is NULL", i);
    if (ctxs[i]->device != p->device) return fail(FGPU_EINVAL, "plan spans devices");
    maxth = std::max(maxth, ctxs[i]->ntheta);
    if (ctxs[i]->mode != ctxs[0]->mode) return fail(FGPU_EINVAL, "plan mixes trailing-update modes");
    p->ctxs.push_back(ctxs[i]);
  }
  if (ldtheta < maxth) return fail(FGPU_EINVAL, "ldtheta=%d < max nparams %d", ldtheta, maxth);
  // the couplings' row-tile order packs (problem << 16 | row tile) into a
  // non-negative int (a negative entry ends a CTA's work)
  if (ctxs[0]->mode == 1 && nprob > 32767)
    return fail(FGPU_EINVAL, "a tensor-core plan holds at most 32767 problems (%d given)", nprob);
  p->ldtheta = ldtheta;
  p->mode = ctxs[0]->mode;
  CK(cudaSetDevice(p->device));
  // waves under the device-memory budget
  std::vector<size_t> bytes(nprob);
  for (int i = 0; i < nprob; ++i) bytes[i] = workspace_bytes(ctxs[i]);
  std::vector<std::vector<int>> groups;
  int rc = plan_waves(bytes, plan_memory_budget(), groups);
  if (rc) return rc;
  for (const auto& g : groups) {
    PlanWave w;
    w.first = (int)p->order.size();
    w.count = (int)g.size();
    for (int i : g) {
      p->order.push_back(i);
      w.bytes += bytes[i];
      w.max_nsteps = std::max(w.max_nsteps, ctxs[i]->nsteps);
      w.max_nplanes = std::max(w.max_nplanes, ctxs[i]->spec.nplanes);
    }
    p->arena_bytes = std::max(p->arena_bytes, w.bytes);
    p->waves.push_back(w);
  }
  // from here on, a failure destroys the partly built plan
  auto bail = [&](int r) {
    fgpu_plan_destroy(p.release());
    return r;
  };
#define PL_CK(call)                                                                            \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      cudaGetLastError();                                                                      \
      return bail(fail(e_ == cudaErrorMemoryAllocation ? FGPU_ENOMEM : FGPU_ECUDA, "%s: %s", #call, \
                       cudaGetErrorString(e_)));                                               \
    }                                                                                          \
  } while (0)
  auto track_alloc = [&](void** dst, size_t n) -> cudaError_t {
    cudaError_t e = cudaMalloc(dst, n);
    if (e == cudaSuccess) p->allocations.push_back(*dst);
    return e;
  };
  PL_CK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  PL_CK(track_alloc((void**)&p->theta_d, sizeof(double) * (size_t)nprob * ldtheta));
  PL_CK(track_alloc((void**)&p->ll_d, sizeof(double) * nprob));
  PL_CK(track_alloc((void**)&p->info_d, sizeof(int) * nprob));
  PL_CK(track_alloc((void**)&p->status_all, sizeof(int) * 4 * nprob));
  PL_CK(track_alloc((void**)&p->probs_d, sizeof(Prob) * nprob));
  unsigned char* arena = nullptr;
  PL_CK(track_alloc((void**)&arena, p->arena_bytes));
  unsigned char* tmaps = nullptr;
  if (p->mode == 1) PL_CK(track_alloc((void**)&tmaps, (size_t)512 * nprob));
  PL_CK(cudaMallocHost(&p->h_theta, sizeof(double) * (size_t)nprob * ldtheta));
  PL_CK(cudaMallocHost(&p->h_ll, sizeof(double) * nprob));
  PL_CK(cudaMallocHost(&p->h_info, sizeof(int) * nprob));
  p->probs_h.resize(nprob);
  for (const PlanWave& w : p->waves) {
    size_t off = 0;  // every wave starts at the arena's base
    for (int k = w.first; k < w.first + w.count; ++k) {
      const int i = p->order[k];
      Workspace ws;
      off += layout_workspace(ctxs[i], arena + off, ws);
      ws.status = p->status_all + 4 * k;
      if (p->mode == 1) {
        ws.tmaps = tmaps + (size_t)512 * k;
        if ((rc = write_tmaps(ctxs[i], ws, ws.tmaps)) != 0) return bail(rc);
      }
      fill_prob(p->probs_h[k], ctxs[i], p->theta_d + (size_t)i * ldtheta, ws);
      p->probs_h[k].ll_dst = p->ll_d + i;
      p->probs_h[k].info_dst = p->info_d + i;
    }
  }
  PL_CK(cudaMemcpy(p->probs_d, p->probs_h.data(), sizeof(Prob) * nprob, cudaMemcpyHostToDevice));
  if (p->mode == 1) {
    for (PlanWave& w : p->waves) {
      std::vector<int> nts, tcs;
      for (int k = w.first; k < w.first + w.count; ++k) {
        nts.push_back(ctxs[p->order[k]]->nt128);
        tcs.push_back(ctxs[p->order[k]]->spec.tc_build);
      }
      if ((rc = build_sched(nts, tcs, w.sched, &p->allocations)) != 0) return bail(rc);
    }
  }
#undef PL_CK
  if ((rc = capture_plan(p.get(), &p->graph, &p->graph_kernels, nullptr)) != 0) return bail(rc);
  *out = p.release();
  return 0;
}

void fgpu_plan_destroy(fgpu_plan* p) {
  if (!p) return;
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  if (p->graph) cudaGraphExecDestroy(p->graph);
  if (p->prof) {
    p->prof->clear();
    delete p->prof;
  }
  for (void* q : p->allocations) cudaFree(q);
  for (PlanWave& w : p->waves) free_sched_sync(w.sched);
  if (p->h_theta) cudaFreeHost(p->h_theta);
  if (p->h_ll) cudaFreeHost(p->h_ll);
  if (p->h_info) cudaFreeHost(p->h_info);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

int fgpu_plan_partition(const long long* bytes, int n, long long budget, int* wave_of, int* nwaves) {
  t_err.clear();
  if (!bytes || n < 1 || !wave_of || !nwaves || budget < 0) return fail(FGPU_EINVAL, "bad partition arguments");
  std::vector<size_t> b(n);
  for (int i = 0; i < n; ++i) {
    if (bytes[i] < 0) return fail(FGPU_EINVAL, "bytes[%d] is negative", i);
    b[i] = (size_t)bytes[i];
  }
  std::vector<std::vector<int>> groups;
  int rc = plan_waves(b, (size_t)budget, groups);
  if (rc) return rc;
  for (size_t w = 0; w < groups.size(); ++w)
    for (int i : groups[w]) wave_of[i] = (int)w;
  *nwaves = (int)groups.size();
  return 0;
}

int fgpu_plan_waves(const fgpu_plan* p, int* nwaves, long long* arena_bytes) {
  t_err.clear();
  if (!p || !nwaves || !arena_bytes) return fail(FGPU_EINVAL, "NULL argument");
  *nwaves = (int)p->waves.size();
  *arena_bytes = (long long)p->arena_bytes;
  return 0;
}

int fgpu_plan_set_profiling(fgpu_plan* p, int enable) {
  t_err.clear();
  if (!p) return fail(FGPU_EINVAL, "plan is NULL");
  if (enable < 0 || enable > 2) return fail(FGPU_EINVAL, "profiling mode must be 0, 1 or 2");
  CK(cudaSetDevice(p->device));
  std::lock_guard<std::mutex> lk(p->mu);
  CK(cudaStreamSynchronize(p->stream));
  if (p->prof) {
    p->prof->clear();
    delete p->prof;
    p->prof = nullptr;
  }
  if (enable) {
    p->prof = new StageEvents();
    if (enable == 2) p->prof->only = 3;  // the trailing update alone: two event nodes per step
  }
  cudaGraphExec_t g = nullptr;
  long long nk = 0;
  int rc = capture_plan(p, &g, &nk, p->prof);
  if (rc) return rc;
  if (p->graph) cudaGraphExecDestroy(p->graph);
  p->graph = g;
  p->graph_kernels = nk;
  return 0;
}

int fgpu_plan_stage_times(fgpu_plan* p, double* ms, int* count) {
  t_err.clear();
  if (!p || !ms || !count) return fail(FGPU_EINVAL, "NULL argument");
  if (!p->prof) return fail(FGPU_EINVAL, "profiling is not enabled on this plan");
  CK(cudaSetDevice(p->device));
  for (int k = 0; k < FGPU_NSTAGES; ++k) {
    ms[k] = 0.0;
    count[k] = 0;
  }
  for (size_t i = 0; i < p->prof->stage.size(); ++i) {
    float t = 0.f;
    CK(cudaEventSynchronize(p->prof->ev[2 * i + 1]));
    CK(cudaEventElapsedTime(&t, p->prof->ev[2 * i], p->prof->ev[2 * i + 1]));
    ms[p->prof->stage[i]] += t;
    count[p->prof->stage[i]] += 1;
  }
  return 0;
}

int fgpu_plan_run_device(fgpu_plan* p, const double* theta_dev, double* ll_dev, int* info_dev, void* stream) {
  t_err.clear();
  if (!p) return fail(FGPU_EINVAL, "plan is NULL");
  CK(cudaSetDevice(p->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
  std::lock_guard<std::mutex> lk(p->mu);
  if (theta_dev && theta_dev != p->theta_d)
    CK(cudaMemcpyAsync(p->theta_d, theta_dev, sizeof(double) * (size_t)p->nprob * p->ldtheta,
                       cudaMemcpyDeviceToDevice, s));
  CK(cudaGraphLaunch(p->graph, s));
  t_launches = p->graph_kernels;
  if (ll_dev && ll_dev != p->ll_d)
    CK(cudaMemcpyAsync(ll_dev, p->ll_d, sizeof(double) * p->nprob, cudaMemcpyDeviceToDevice, s));
  if (info_dev && info_dev != p->info_d)
    CK(cudaMemcpyAsync(info_dev, p->info_d, sizeof(int) * p->nprob, cudaMemcpyDeviceToDevice, s));
  return 0;
}

int fgpu_plan_run(fgpu_plan* p, const double* theta_host, double* ll_host, int* info_host) {
  t_err.clear();
  if (!p || !theta_host || !ll_host || !info_host) return fail(FGPU_EINVAL, "NULL argument");
  CK(cudaSetDevice(p->device));
  std::lock_guard<std::mutex> lk(p->mu);
  const size_t tb = sizeof(double) * (size_t)p->nprob * p->ldtheta;
  memcpy(p->h_theta, theta_host, tb);
  CK(cudaMemcpyAsync(p->theta_d, p->h_theta, tb, cudaMemcpyHostToDevice, p->stream));
  CK(cudaGraphLaunch(p->graph, p->stream));
  t_launches = p->graph_kernels;
  CK(cudaMemcpyAsync(p->h_ll, p->ll_d, sizeof(double) * p->nprob, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaMemcpyAsync(p->h_info, p->info_d, sizeof(int) * p->nprob, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
  memcpy(ll_host, p->h_ll, sizeof(double) * p->nprob);
  memcpy(info_host, p->h_info, sizeof(int) * p->nprob);
  for (int i = 0; i < p->nprob; ++i) {
    if (info_host[i] == -1) return fail(FGPU_ETIMEOUT, "problem %d: a bounded wait in a kernel gave up", i);
    if (info_host[i] < 0) return fail(FGPU_ECUDA, "problem %d: panel value outside its row scale bound", i);
  }
  return 0;
}

int fgpu_loglik_batch(fgpu_ctx* const* ctxs, int nprob, const double* const* theta, double* ll, int* info) {
  t_err.clear();
  if (!ctxs || !theta || !ll || !info || nprob < 1) return fail(FGPU_EINVAL, "bad batch arguments");
  std::vector<fgpu_ctx*> key(ctxs, ctxs + nprob);
  int maxth = 0;
  for (int i = 0; i < nprob; ++i) {
    if (!ctxs[i] || !theta[i]) return fail(FGPU_EINVAL, "NULL entry %d", i);
    maxth = std::max(maxth, ctxs[i]->ntheta);
  }
  std::shared_ptr<fgpu_plan> sp;
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
      sp = it->second.plan;
      it->second.used = ++g_plan_clock;
    }
  }
  if (!sp) {
    fgpu_plan* raw = nullptr;
    int rc = fgpu_plan_create(&raw, ctxs, nprob, std::max(maxth, 1));
    if (rc) return rc;
    sp = std::shared_ptr<fgpu_plan>(raw, fgpu_plan_destroy);
    std::vector<std::shared_ptr<fgpu_plan>> drop;  // evicted plans, destroyed outside the lock
    std::lock_guard<std::mutex> lk(g_plan_mu);
    CachedPlan& e = g_plans[key];
    if (e.plan) drop.push_back(e.plan);  // another thread built the same plan meanwhile
    e.plan = sp;
    e.used = ++g_plan_clock;
    while (g_plans.size() > plan_cache_limit()) {
      auto lru = g_plans.begin();
      for (auto it = g_plans.begin(); it != g_plans.end(); ++it)
        if (it->second.used < lru->second.used) lru = it;
      drop.push_back(std::move(lru->second.plan));
      g_plans.erase(lru);
    }
  }
  fgpu_plan* p = sp.get();
  std::vector<double> th((size_t)nprob * p->ldtheta, 0.0);
  for (int i = 0; i < nprob; ++i) {
    for (int k = 0; k < ctxs[i]->ntheta; ++k) {
      if (!std::isfinite(theta[i][k])) return fail(FGPU_EINVAL, "theta[%d][%d] is not finite", i, k);
      th[(size_t)i * p->ldtheta + k] = theta[i][k];
    }
  }
  return fgpu_plan_run(p, th.data(), ll, info);
}

}  // extern "C"

// Hooks for other translation units of the library: the spec compiler and the
// thread-local error channel behind fgpu_last_error().
namespace fgpu {
int internal_compile_spec(const int* kspec, int nkspec, int d, Spec& sp, std::vector<int>& plane_dim,
                          std::vector<int>& plane_kind) {
  t_err.clear();
  return compile_spec(kspec, nkspec, d, sp, plane_dim, plane_kind);
}
int internal_fail(int code, const char* msg) { return fail(code, "%s", msg); }
void internal_clear_error() {
  t_err.clear();
  t_launches = 0;
}
void internal_add_launches(long long n) { t_launches += n; }
}  // namespace fgpu
