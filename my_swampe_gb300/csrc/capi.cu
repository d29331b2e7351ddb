// C ABI of libswampe_gb300: plan lifetime, launch decomposition and the
// step loop.  See include/swampe_gb300.h for the contract of each symbol.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <new>
#include <type_traits>
#include "swp_internal.h"

using namespace swp;

struct GraphEntry {
  std::vector<uint64_t> key;
  cudaGraphExec_t exec = nullptr;
  uint64_t last_use = 0;
};

struct swp_plan {
  int precision = SWP_FP64;
  int ng = 0;
  cudaStream_t cap_stream = nullptr;     // private stream used only for graph capture
  std::vector<GraphEntry> graphs;        // small LRU cache of instantiated step graphs
  uint64_t use_clock = 0;
  bool graphs_enabled = true;
  GroupGeom geom[MAXG];
  int M[MAXG] = {}, B[MAXG] = {}, MT[MAXG] = {}, JB[MAXG] = {};
  size_t spec_smem = 0;
  size_t spec_adj_smem = 0;
  size_t grid_smem[NGRIDMODE] = {};
  // tensor-core Legendre kernels of the FP32 step: tc[g] for the groups that
  // run them (M = 42, 63 or 106), use_tc if any group does
  bool use_tc = false;
  bool tc[MAXG] = {};
  float* tcbasis[MAXG] = {};
  float* tcbasis_adj[MAXG] = {};
  void* coefmem[MAXG] = {};              // per-call coefficient tables (CoefTables) of each group
  int* d_err = nullptr;                  // device error word set by bounded waits that ran out
  SchedCounter* d_sched = nullptr;       // persistent-launch counters: one per group chain, one for joint launches
  uint32_t tc_wait_limit = TC_WAIT_LIMIT_DEFAULT;  // mbarrier polls before a tensor-core wait gives up
  // groups run concurrently: each group's step chain on its own stream (forked
  // from and joined to the caller's), so that one group's latency-bound kernels
  // overlap another's; gmask restricts launches to the groups of one chain
  bool concurrent = false;
  unsigned gmask = ~0u;
  cudaStream_t side[MAXG] = {};
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t ev_join[MAXG] = {};
  std::string err;
};

namespace {

int fail(swp_plan* p, int code, const std::string& msg) {
  if (p) p->err = msg;
  return code;
}

int cuda_check(swp_plan* p, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return SWP_OK;
  return fail(p, SWP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// whether group g takes part in the launches being built (see swp_plan::gmask)
inline bool active(const swp_plan* p, int g) { return (p->gmask >> g) & 1u; }

// Run body(stream) once for all groups, or -- on a concurrent plan with more
// than one group -- once per group on that group's stream, forked from `cs`
// and joined back into it (inside a graph capture the chains become parallel
// branches of the graph).
template <typename F>
int per_group_streams(swp_plan* p, cudaStream_t cs, F body) {
  if (!p->concurrent || p->ng < 2) return body(cs);
  cudaError_t e = cudaSuccess;
  if (!p->ev_fork) e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming);
  for (int g = 0; g < p->ng && e == cudaSuccess; ++g) {
    if (!p->side[g]) e = cudaStreamCreateWithFlags(&p->side[g], cudaStreamNonBlocking);
    if (e == cudaSuccess && !p->ev_join[g]) e = cudaEventCreateWithFlags(&p->ev_join[g], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) return cuda_check(p, e, "concurrent group streams");
  if (int rc = cuda_check(p, cudaEventRecord(p->ev_fork, cs), "fork")) return rc;
  int rc = SWP_OK;
  for (int g = 0; g < p->ng && rc == SWP_OK; ++g) {
    rc = cuda_check(p, cudaStreamWaitEvent(p->side[g], p->ev_fork, 0), "fork wait");
    if (rc) break;
    p->gmask = 1u << g;
    rc = body(p->side[g]);
    p->gmask = ~0u;
    if (rc) break;
    rc = cuda_check(p, cudaEventRecord(p->ev_join[g], p->side[g]), "join");
    if (rc) break;
    rc = cuda_check(p, cudaStreamWaitEvent(cs, p->ev_join[g], 0), "join wait");
  }
  p->gmask = ~0u;
  return rc;
}

template <typename T>
CoefTables<T> plan_coefs(const swp_plan* p, int g) {
  CoefTables<T> C;
  C.carve((T*)p->coefmem[g], p->M[g], p->B[g], p->geom[g].J);
  return C;
}

// Refresh the coefficient tables from the members' parameters: first launch of
// every call that runs step kernels.
template <typename T>
int update_coefs(swp_plan* p, const swp_group_state* st, cudaStream_t s, const swp_group_tangent* tan = nullptr) {
  for (int g = 0; g < p->ng; ++g) {
    if (!active(p, g)) continue;
    cudaError_t e = launch_coefs<T>(st[g].params, p->geom[g].onemu2, p->M[g], p->B[g], p->geom[g].J,
                                    plan_coefs<T>(p, g), s, tan ? tan[g].dparams : nullptr);
    if (e != cudaSuccess) return cuda_check(p, e, "coefficient kernel launch");
  }
  return SWP_OK;
}

// Persistent scheduling of a SIMT Legendre launch: the groups in order of
// decreasing truncation (their units cost the most), and the counter of the
// chain the launch belongs to (a group's own stream, or the joint launches).
template <typename T>
void set_schedule(const swp_plan* p, SpecLaunch<T>& L) {
  int order[MAXG];
  for (int g = 0; g < p->ng; ++g) order[g] = g;
  std::stable_sort(order, order + p->ng, [&](int a, int b) { return p->M[a] > p->M[b]; });
  int acc = 0;
  for (int k = 0; k < p->ng; ++k) {
    L.sorder[k] = order[k];
    L.sprefix[k] = acc;
    acc += (p->M[order[k]] + 1) * L.grp[order[k]].ntb;
  }
  L.sprefix[p->ng] = acc;
  int chain = MAXG;
  if (p->concurrent && p->ng > 1 && __builtin_popcount(p->gmask & ((1u << p->ng) - 1)) == 1)
    chain = __builtin_ctz(p->gmask);
  L.sched = p->d_sched ? p->d_sched + chain : nullptr;
}

template <typename T>
SpecLaunch<T> make_spec(const swp_plan* p, const swp_group_state* st, int& nblocks) {
  SpecLaunch<T> L;
  memset(&L, 0, sizeof(L));
  L.ng = p->ng;
  int acc = 0;
  for (int g = 0; g < p->ng; ++g) {
    SpecGroup<T>& G = L.grp[g];
    G.g = p->geom[g].view<T>();
    G.B = active(p, g) ? p->B[g] : 0;  // an inactive group gets no CTAs
    G.MT = p->MT[g];
    G.ntb = (G.B + G.MT - 1) / G.MT;
    G.four = (typename cplx<T>::type*)st[g].fourier;
    G.four_out = G.four;
    G.par = st[g].params;
    G.member = st[g].member;
    G.diag = st[g].diag;
    CoefTables<T> C = plan_coefs<T>(p, g);
    G.nco = C.nco;
    G.jco = C.jco;
    G.djco = C.djco;
    G.mco = C.mco;
    L.prefix[g] = acc;
    acc += (p->M[g] + 1) * G.ntb;
  }
  L.prefix[p->ng] = acc;
  nblocks = acc;
  set_schedule(p, L);
  return L;
}

template <typename T>
GridLaunch<T> make_grid(const swp_plan* p, const swp_group_state* st, int& nblocks) {
  GridLaunch<T> L;
  memset(&L, 0, sizeof(L));
  L.ng = p->ng;
  int acc = 0;
  for (int g = 0; g < p->ng; ++g) {
    GridGroup<T>& G = L.grp[g];
    G.g = p->geom[g].view<T>();
    G.B = active(p, g) ? p->B[g] : 0;  // an inactive group gets no CTAs
    G.JB = p->JB[g];
    G.njb = p->geom[g].J / G.JB;
    G.four = (typename cplx<T>::type*)st[g].fourier;
    G.resid = (T*)st[g].resid;
    G.par = st[g].params;
    G.member = st[g].member;
    G.diag = st[g].diag;
    L.prefix[g] = acc;
    acc += G.B * G.njb;
  }
  L.prefix[p->ng] = acc;
  nblocks = acc;
  return L;
}

StepCfg make_cfg(const swp_flags* f) {
  StepCfg c;
  memset(&c, 0, sizeof(c));
  c.scheme = f->scheme;
  c.raw = f->raw_filter != 0;
  // relaxation and drag are implicit only where the physical forcing is on
  // (model.py:912-914: forcflag and test is None)
  c.si_relax = f->scheme == 2 && f->forcflag && f->test == 0;
  c.forcflag = f->forcflag;
  c.diffflag = f->diffflag;
  c.test = f->test;
  c.diagnostics = f->diagnostics;
  c.blowup = f->blowup;
  return c;
}

// The incremental form needs a band-limited Fourier curr carry: true after a
// member's first modified-Euler step, but the RAW filter mixes the initial
// condition's (not band-limited) Fourier coefficients back into it.
bool step_incremental(const swp_plan* p, const swp_flags* f, int t) {
  return p->precision == SWP_FAST && f->scheme == 0 && !f->raw_filter && t > f->t_start;
}

// Whether group g runs the tensor-core form of the forward (adjoint = false) or
// adjoint Legendre kernel.
bool tc_group(const swp_plan* p, int g, bool adjoint) {
  return p->tc[g] && (!adjoint || spec_tc_adj_supported(p->M[g]));
}

// Tensor-core launches of one step: one launch per truncation present (42, 63,
// 106), each over the groups of that truncation (the others get no CTAs).
template <typename Launch>
cudaError_t launch_tc_per_truncation(const swp_plan* p, const SpecLaunch<float>& LS, float* const* bases,
                                     bool adjoint, Launch launch) {
  const int mt = spec_tc_members_per_cta();
  for (int Mt : {42, 63, 106}) {
    SpecLaunch<float> LT = LS;
    int acc = 0;
    TcBasis tb;
    memset(&tb, 0, sizeof(tb));
    tb.wait_limit = p->tc_wait_limit;
    bool any = false;
    for (int g = 0; g < p->ng; ++g) {
      if (p->M[g] != Mt || !tc_group(p, g, adjoint)) LT.grp[g].B = 0;
      LT.grp[g].MT = mt;
      LT.grp[g].ntb = (LT.grp[g].B + mt - 1) / mt;
      LT.prefix[g] = acc;
      acc += (p->M[g] + 1) * LT.grp[g].ntb;
      tb.p[g] = bases[g];
      any = any || (p->M[g] == Mt && LT.grp[g].B > 0);
    }
    LT.prefix[p->ng] = acc;
    if (!any) continue;
    cudaError_t e = launch(Mt, LT, acc, tb);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The SIMT launch of the groups that do not run the tensor-core kernels (the
// others get no CTAs); returns the block count through nb.
template <typename T>
SpecLaunch<T> simt_only(const swp_plan* p, const SpecLaunch<T>& LS, bool adjoint, int& nb) {
  SpecLaunch<T> L = LS;
  int acc = 0;
  for (int g = 0; g < p->ng; ++g) {
    if (tc_group(p, g, adjoint)) L.grp[g].B = 0;
    L.grp[g].ntb = (L.grp[g].B + L.grp[g].MT - 1) / L.grp[g].MT;
    L.prefix[g] = acc;
    acc += (p->M[g] + 1) * L.grp[g].ntb;
  }
  L.prefix[p->ng] = acc;
  nb = acc;
  set_schedule(p, L);
  return L;
}

// The Legendre kernel of a modified-Euler step: tcgen05 (3xTF32) on the FP32
// path when the plan packed the tensor-core basis, the SIMT kernel otherwise.
template <typename T>
cudaError_t launch_step_spec(const swp_plan* p, const SpecLaunch<T>& LS, int nbs, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    if (p->use_tc && LS.mode == 0 && LS.cfg.scheme == 0 && !LS.cfg.tl_filter) {
      cudaError_t e = launch_tc_per_truncation(p, LS, p->tcbasis, false,
                                               [&](int Mt, const SpecLaunch<float>& LT, int n, const TcBasis& tb) {
                                                 return launch_spec_tc(Mt, LT, n, tb, p->d_err, s);
                                               });
      int nb = 0;
      SpecLaunch<float> LR = simt_only(p, LS, false, nb);
      if (e == cudaSuccess && nb > 0) e = launch_spec<T>(LR, nb, p->spec_smem, s);
      return e;
    }
  }
  return launch_spec<T>(LS, nbs, p->spec_smem, s);
}

// The Legendre adjoint of a modified-Euler step: tcgen05 on the FP32 path when
// the plan packed the tensor-core basis, the SIMT kernel otherwise.
template <typename T>
cudaError_t launch_step_spec_adj(const swp_plan* p, const SpecLaunch<T>& LS, int nbs, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value) {
    if (p->use_tc && LS.cfg.scheme == 0) {
      cudaError_t e = launch_tc_per_truncation(p, LS, p->tcbasis_adj, true,
                                               [&](int Mt, const SpecLaunch<float>& LT, int n, const TcBasis& tb) {
                                                 return launch_spec_adj_tc(Mt, LT, n, tb, p->d_err, s);
                                               });
      int nb = 0;
      SpecLaunch<float> LR = simt_only(p, LS, true, nb);
      if (e == cudaSuccess && nb > 0) e = launch_spec_adj<T>(LR, nb, p->spec_adj_smem, s);
      return e;
    }
  }
  return launch_spec_adj<T>(LS, nbs, p->spec_adj_smem, s);
}

// Launch nsteps steps.  In place on st[g].fourier, or -- when `slots` is given --
// out of place: step k reads slot k and writes slot k+1 (slot stride `sstride`
// complex elements), which keeps every intermediate state of a window.
template <typename T>
int forward_steps(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps, int row0,
                  int write_prev_last, void* const* slots, cudaStream_t s) {
  typedef typename cplx<T>::type T2;
  int nbs = 0, nbg = 0;
  SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LS.mode = 0;
  LG.mode = GM_STEP;
  StepCfg cfg = make_cfg(f);
  if (nsteps > 0) {
    int rc = update_coefs<T>(p, st, s);
    if (rc) return rc;
  }
  for (int k = 0; k < nsteps; ++k) {
    int t = t0 + k;
    cfg.step = row0 + k;
    cfg.ra_mode = (f->modalflag && t > 2) ? 2 : 1;
    // the semi-implicit scheme keeps its lagged remainders in the prev slots
    cfg.write_prev = f->scheme != 2 && ((f->scheme == 1) || (write_prev_last && k == nsteps - 1));
    cfg.si_lag_init = f->scheme == 2 && t == f->t_start;
    cfg.incremental = step_incremental(p, f, t) ? 1 : 0;
    LS.cfg = cfg;
    LG.cfg = cfg;
    for (int g = 0; g < p->ng; ++g) {
      size_t PS = (size_t)p->B[g] * p->geom[g].J * p->geom[g].I;
      LG.grp[g].hist = st[g].hist ? (T*)st[g].hist + (size_t)(row0 + k) * 5 * PS : nullptr;
      if (slots) {
        size_t ss = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J;
        LS.grp[g].four = (T2*)slots[g] + (size_t)k * ss;
        LS.grp[g].four_out = (T2*)slots[g] + (size_t)(k + 1) * ss;
        LG.grp[g].four = LS.grp[g].four_out;
      }
    }
    cudaError_t e = launch_step_spec<T>(p, LS, nbs, s);
    if (e != cudaSuccess) return cuda_check(p, e, "spectral kernel launch");
    e = launch_grid<T>(LG, nbg, p->grid_smem[GM_STEP], s);
    if (e != cudaSuccess) return cuda_check(p, e, "grid kernel launch");
  }
  return SWP_OK;
}

// Run `body(stream)` through a cached CUDA graph keyed by `key` (captured on the
// plan's private stream, launched on the caller's stream).
template <typename F>
int run_graph(swp_plan* p, const std::vector<uint64_t>& key, F body0, cudaStream_t s) {
  auto body = [&](cudaStream_t cs) { return per_group_streams(p, cs, body0); };
  if (!p->graphs_enabled) return body(s);
  GraphEntry* hit = nullptr;
  for (auto& ge : p->graphs)
    if (ge.key == key) { hit = &ge; break; }
  if (!hit) {
    if (!p->cap_stream) {
      cudaError_t e = cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking);
      if (e != cudaSuccess) return cuda_check(p, e, "capture stream");
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_check(p, e, "graph capture begin");
    int rc = body(p->cap_stream);
    e = cudaStreamEndCapture(p->cap_stream, &graph);
    if (rc != SWP_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (e != cudaSuccess) return cuda_check(p, e, "graph capture end");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_check(p, e, "graph instantiate");
    if (p->graphs.size() >= 16) {  // evict the least recently used graph
      size_t lru = 0;
      for (size_t i = 1; i < p->graphs.size(); ++i)
        if (p->graphs[i].last_use < p->graphs[lru].last_use) lru = i;
      cudaGraphExecDestroy(p->graphs[lru].exec);
      p->graphs.erase(p->graphs.begin() + lru);
    }
    GraphEntry ge;
    ge.key = key;
    ge.exec = exec;
    p->graphs.push_back(ge);
    hit = &p->graphs.back();
  }
  hit->last_use = ++p->use_clock;
  return cuda_check(p, cudaGraphLaunch(hit->exec, s), "graph launch");
}

void key_flags(std::vector<uint64_t>& k, const swp_flags* f) {
  k.push_back((uint64_t)f->scheme | ((uint64_t)f->forcflag << 4) | ((uint64_t)f->diffflag << 8) |
              ((uint64_t)f->modalflag << 12) | ((uint64_t)f->test << 16) | ((uint64_t)f->diagnostics << 20) |
              ((uint64_t)(f->raw_filter != 0) << 24));
  uint64_t bu;
  memcpy(&bu, &f->blowup, 8);
  k.push_back(bu);
  k.push_back((uint64_t)(int64_t)f->t_start);
}

void key_state(std::vector<uint64_t>& k, const swp_plan* p, const swp_group_state* st) {
  for (int g = 0; g < p->ng; ++g) {
    k.push_back((uint64_t)st[g].fourier); k.push_back((uint64_t)st[g].resid); k.push_back((uint64_t)st[g].params);
    k.push_back((uint64_t)st[g].member); k.push_back((uint64_t)st[g].diag); k.push_back((uint64_t)st[g].hist);
  }
}

template <typename T>
int forward_impl(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps,
                 int row0, int write_prev_last, cudaStream_t s) {
  if (nsteps < 4) return forward_steps<T>(p, st, f, t0, nsteps, row0, write_prev_last, nullptr, s);
  bool plain = true;  // no per-step rows (diagnostics, history)
  for (int g = 0; g < p->ng; ++g) plain = plain && !st[g].diag && !st[g].hist;
  constexpr int WIN = 128;
  if (plain && nsteps > 2 * WIN) {
    // A long run is a few step windows, each a captured graph.  From t_steady on
    // every step launches the same kernels with the same arguments (the step
    // index only selects the projected first step, the filter's start at t = 3
    // and the semi-implicit lag initialisation), so one window graph serves the
    // whole run instead of a graph of every step.
    const int t_steady = std::max(3, f->t_start + 1);
    const int head = std::min(nsteps, std::max(0, t_steady - t0));
    int done = 0;
    if (head > 0) {
      if (int rc = forward_impl<T>(p, st, f, t0, head, row0, write_prev_last && head == nsteps, s)) return rc;
      done = head;
    }
    while (done < nsteps) {
      const int n = std::min(WIN, nsteps - done);
      const int wpl = (write_prev_last && done + n == nsteps) ? 1 : 0;
      const int tw = t0 + done;
      std::vector<uint64_t> key = {5, (uint64_t)n, (uint64_t)wpl};
      key_flags(key, f);
      key_state(key, p, st);
      int rc = n < 4 ? forward_steps<T>(p, st, f, tw, n, row0, wpl, nullptr, s)
                     : run_graph(p, key, [&](cudaStream_t cs) {
                         return forward_steps<T>(p, st, f, tw, n, row0, wpl, nullptr, cs);
                       }, s);
      if (rc) return rc;
      done += n;
    }
    return SWP_OK;
  }
  std::vector<uint64_t> key = {1, (uint64_t)t0, (uint64_t)nsteps, (uint64_t)row0, (uint64_t)write_prev_last};
  key_flags(key, f);
  key_state(key, p, st);
  return run_graph(p, key, [&](cudaStream_t cs) {
    return forward_steps<T>(p, st, f, t0, nsteps, row0, write_prev_last, nullptr, cs);
  }, s);
}

// ------------------------------------------------------------ tangent-linear
// The tangent state uses the primal's parameters, coefficient tables and
// residual weights (the filter recursion does not depend on the state); only
// its Fourier carries and residuals are its own.
static void tangent_states(const swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan,
                           swp_group_state* tst) {
  for (int g = 0; g < p->ng; ++g) {
    tst[g] = st[g];
    tst[g].fourier = tan[g].fourier;
    tst[g].resid = tan[g].resid;
    tst[g].diag = nullptr;
    tst[g].hist = nullptr;
  }
}

template <typename T>
int tangent_init_impl(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, void* const* phys,
                      void* const* dphys, const swp_flags* f, cudaStream_t s) {
  swp_group_state tst[MAXG];
  tangent_states(p, st, tan, tst);
  size_t es = sizeof(typename cplx<T>::type);
  for (int g = 0; g < p->ng; ++g) {
    size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
    int rc = cuda_check(p, cudaMemsetAsync(tan[g].fourier, 0, bytes, s), "tangent state clear");
    if (rc) return rc;
    // the initial residual weights are constants
    rc = cuda_check(p, cudaMemsetAsync(tan[g].dweights, 0, 2 * sizeof(double) * p->B[g], s),
                    "tangent weights clear");
    if (rc) return rc;
  }
  int nbg = 0;
  GridLaunch<T> LG = make_grid<T>(p, tst, nbg);
  LG.mode = GM_TL_INIT;
  LG.cfg = make_cfg(f);
  LG.cfg.diagnostics = 0;
  for (int g = 0; g < p->ng; ++g) {
    LG.grp[g].phys_in = (const T*)dphys[g];
    LG.grp[g].phys_p = (const T*)phys[g];
    LG.grp[g].dpar = tan[g].dparams;
  }
  return cuda_check(p, launch_grid<T>(LG, nbg, p->grid_smem[GM_TL_INIT], s), "tangent init launch");
}

// One window of primal + tangent steps.  Per step: the tangent Legendre step
// (it reads the primal state before the step), the primal Legendre step, the
// primal grid step, then the tangent grid step (linearised about the new
// primal level).  Along tangents of the filter weights (alpha, williams_alpha)
// the filtered levels also move by the weights' tangents times the primal
// displacement mid - 2 curr + new, which exists only inside the primal step:
// that step (then on the SIMT kernel) adds those terms to the tangent carries
// and advances the tangents of the residual weights.
template <typename T>
int tangent_steps(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, const swp_flags* f, int t0,
                  int nsteps, cudaStream_t s) {
  swp_group_state tst[MAXG];
  tangent_states(p, st, tan, tst);
  int nbs = 0, nbg = 0;
  SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
  SpecLaunch<T> LT = make_spec<T>(p, tst, nbs);
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  GridLaunch<T> LGT = make_grid<T>(p, tst, nbg);
  LS.mode = 0;
  LT.mode = 3;
  LG.mode = GM_STEP;
  LGT.mode = GM_TL_STEP;
  for (int g = 0; g < p->ng; ++g) {
    LT.grp[g].four_p = (const typename cplx<T>::type*)st[g].fourier;
    LT.grp[g].dpar = tan[g].dparams;
    LS.grp[g].four_t = (typename cplx<T>::type*)tan[g].fourier;
    LS.grp[g].dpar = tan[g].dparams;
    LS.grp[g].dw = tan[g].dweights;
    LGT.grp[g].primal = (const typename cplx<T>::type*)st[g].fourier;
    LGT.grp[g].dpar = tan[g].dparams;
    LGT.grp[g].resid_p = (const T*)st[g].resid;
    LGT.grp[g].dw = tan[g].dweights;
    LG.grp[g].hist = nullptr;
  }
  StepCfg cfg = make_cfg(f);
  cfg.diagnostics = 0;
  // the semi-implicit solve depends on taurad, taudrag, Phibar: its tangent always takes the coefficient pass
  cfg.tl_coef = f->scheme == 2;
  for (int g = 0; g < p->ng; ++g) cfg.tl_coef |= tan[g].coef_tangents != 0;
  if (nsteps > 0) {
    int rc = update_coefs<T>(p, st, s, tan);
    if (rc) return rc;
  }
  for (int k = 0; k < nsteps; ++k) {
    int t = t0 + k;
    cfg.step = k;
    cfg.ra_mode = (f->modalflag && t > 2) ? 2 : 1;
    // as forward_steps: the semi-implicit scheme keeps its lagged remainders in the prev slots
    cfg.write_prev = f->scheme != 2 && (f->scheme == 1 || k == nsteps - 1);
    cfg.si_lag_init = f->scheme == 2 && t == f->t_start;
    cfg.incremental = step_incremental(p, f, t) ? 1 : 0;
    LS.cfg = LT.cfg = LG.cfg = LGT.cfg = cfg;
    LS.cfg.tl_filter = cfg.tl_coef && cfg.ra_mode == 2;
    cudaError_t e = launch_spec<T>(LT, nbs, p->spec_smem, s);
    if (e != cudaSuccess) return cuda_check(p, e, "tangent spectral kernel launch");
    e = launch_step_spec<T>(p, LS, nbs, s);
    if (e != cudaSuccess) return cuda_check(p, e, "spectral kernel launch");
    e = launch_grid<T>(LG, nbg, p->grid_smem[GM_STEP], s);
    if (e != cudaSuccess) return cuda_check(p, e, "grid kernel launch");
    e = launch_grid<T>(LGT, nbg, p->grid_smem[GM_TL_STEP], s);
    if (e != cudaSuccess) return cuda_check(p, e, "tangent grid kernel launch");
  }
  return SWP_OK;
}

template <typename T>
int tangent_forward_impl(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, const swp_flags* f,
                         int t0, int nsteps, cudaStream_t s) {
  if (nsteps < 4) return tangent_steps<T>(p, st, tan, f, t0, nsteps, s);
  std::vector<uint64_t> key = {3, (uint64_t)t0, (uint64_t)nsteps};
  key_flags(key, f);
  key_state(key, p, st);
  for (int g = 0; g < p->ng; ++g) {
    key.push_back((uint64_t)tan[g].fourier);
    key.push_back((uint64_t)tan[g].resid);
    key.push_back((uint64_t)tan[g].dparams);
    key.push_back((uint64_t)tan[g].dweights);
    key.push_back((uint64_t)(tan[g].coef_tangents != 0));
  }
  return run_graph(p, key, [&](cudaStream_t cs) { return tangent_steps<T>(p, st, tan, f, t0, nsteps, cs); }, s);
}

template <typename T>
int init_impl(swp_plan* p, const swp_group_state* st, void* const* phys, const swp_flags* f, cudaStream_t s) {
  int nbg = 0;
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LG.mode = GM_INIT;
  LG.cfg = make_cfg(f);
  for (int g = 0; g < p->ng; ++g) LG.grp[g].phys_in = (const T*)phys[g];
  return cuda_check(p, launch_grid<T>(LG, nbg, p->grid_smem[GM_INIT], s), "init kernel launch");
}

template <typename T>
int output_impl(swp_plan* p, const swp_group_state* st, void* const* out, const swp_flags* f, cudaStream_t s,
                const swp_group_state* primal = nullptr, const swp_group_tangent* tan = nullptr) {
  int nbg = 0;
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LG.mode = GM_OUTPUT;
  LG.cfg = make_cfg(f);
  LG.cfg.diagnostics = 0;
  for (int g = 0; g < p->ng; ++g) {
    LG.grp[g].phys_out = (T*)out[g];
    // tangent output: the residual weights' tangents times the primal residual
    if (primal && tan) {
      LG.grp[g].resid_p = (const T*)primal[g].resid;
      LG.grp[g].dw = tan[g].dweights;
    }
  }
  return cuda_check(p, launch_grid<T>(LG, nbg, p->grid_smem[GM_OUTPUT], s), "output kernel launch");
}

template <typename T>
int winds_impl(swp_plan* p, const swp_group_state* st, void* const* ed, void* const* uv, cudaStream_t s) {
  // model.py:644-666: FFT of eta, delta -> fwd_leg -> invrsUV -> real(ifft)
  int nbg = 0, nbs = 0;
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LG.mode = GM_FWD2;
  for (int g = 0; g < p->ng; ++g) LG.grp[g].phys_in = (const T*)ed[g];
  cudaError_t e = launch_grid<T>(LG, nbg, p->grid_smem[GM_FWD2], s);
  if (e != cudaSuccess) return cuda_check(p, e, "winds forward transform");
  int rc = update_coefs<T>(p, st, s);
  if (rc) return rc;
  SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
  LS.mode = 2;
  e = launch_spec<T>(LS, nbs, p->spec_smem, s);
  if (e != cudaSuccess) return cuda_check(p, e, "winds Legendre kernel");
  LG.mode = GM_WINDS;
  for (int g = 0; g < p->ng; ++g) { LG.grp[g].phys_out = (T*)uv[g]; LG.grp[g].member = nullptr; }
  e = launch_grid<T>(LG, nbg, p->grid_smem[GM_WINDS], s);
  return cuda_check(p, e, "winds inverse transform");
}

// `sweep`: the step is one of an adjoint sweep, whose lambda always comes from
// the Legendre adjoint (or the seed), so the grid adjoint may use its tied
// F / G components (modified Euler; the explicit scheme's are not tied).
// `zeroed`: an earlier step of the same sweep has zeroed the adjoint of U, V
// and of the prev / mid carries (modified Euler: no step input reads them).
template <typename T>
int adjoint_step_impl(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                      const swp_group_adjoint* adj, const swp_flags* f, int t, cudaStream_t s,
                      bool refresh_coefs = true, bool sweep = false, bool zeroed = false) {
  zeroed = zeroed && sweep && f->scheme == 0;
  int nbg = 0, nbs = 0;
  if (refresh_coefs) {
    int rc = update_coefs<T>(p, st_in, s);
    if (rc) return rc;
  }
  GridLaunch<T> LG = make_grid<T>(p, st_out, nbg);
  LG.mode = GM_ADJ_STEP;
  LG.cfg = make_cfg(f);
  LG.cfg.lam_fg_tied = (sweep && f->forcflag && f->test == 0 && f->scheme == 0) ? 1 : 0;
  LG.cfg.adj_zeroed = zeroed ? 1 : 0;
  for (int g = 0; g < p->ng; ++g) {
    LG.grp[g].primal = (const typename cplx<T>::type*)st_out[g].fourier;
    LG.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
    LG.grp[g].lamy = (typename cplx<T>::type*)adj[g].lam_y;
    LG.grp[g].grad = adj[g].grad;
    LG.grp[g].member = nullptr;
  }
  cudaError_t e = launch_grid<T>(LG, nbg, p->grid_smem[GM_ADJ_STEP], s);
  if (e != cudaSuccess) return cuda_check(p, e, "grid adjoint launch");
  SpecLaunch<T> LS = make_spec<T>(p, st_in, nbs);
  LS.mode = 0;
  LS.cfg = make_cfg(f);
  LS.cfg.incremental = step_incremental(p, f, t) ? 1 : 0;
  // the carries of step t, as forward_steps sets them (read by the semi-implicit adjoint)
  LS.cfg.ra_mode = (f->modalflag && t > 2) ? 2 : 1;
  LS.cfg.si_lag_init = f->scheme == 2 && t == f->t_start;
  LS.cfg.adj_zeroed = zeroed ? 1 : 0;
  for (int g = 0; g < p->ng; ++g) {
    LS.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
    LS.grp[g].lamY = (const typename cplx<T>::type*)adj[g].lam_y;
    LS.grp[g].grad = adj[g].grad;
  }
  e = launch_step_spec_adj<T>(p, LS, nbs, s);
  return cuda_check(p, e, "spectral adjoint launch");
}

template <typename T>
int adjoint_seed_impl(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, void* const* dphys,
                      cudaStream_t s) {
  size_t es = sizeof(typename cplx<T>::type);
  for (int g = 0; g < p->ng; ++g) {
    size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
    int rc = cuda_check(p, cudaMemsetAsync(adj[g].lam, 0, bytes, s), "adjoint seed memset");
    if (rc) return rc;
  }
  int nbg = 0;
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LG.mode = GM_ADJ_OUTPUT;
  for (int g = 0; g < p->ng; ++g) {
    LG.grp[g].phys_in = (const T*)dphys[g];
    LG.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
    LG.grp[g].member = nullptr;
  }
  return cuda_check(p, launch_grid<T>(LG, nbg, p->grid_smem[GM_ADJ_OUTPUT], s), "adjoint seed launch");
}

template <typename T>
int adjoint_init_impl(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, void* const* phys_ic,
                      void* const* dic, const swp_flags* f, cudaStream_t s) {
  int nbg = 0;
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LG.mode = GM_ADJ_INIT;
  LG.cfg = make_cfg(f);
  for (int g = 0; g < p->ng; ++g) {
    LG.grp[g].phys_in = (const T*)phys_ic[g];
    LG.grp[g].phys_out = (T*)dic[g];
    LG.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
    LG.grp[g].grad = adj[g].grad;
    LG.grp[g].member = nullptr;
  }
  return cuda_check(p, launch_grid<T>(LG, nbg, p->grid_smem[GM_ADJ_INIT], s), "adjoint init launch");
}

template <typename T>
int adjoint_window_impl(swp_plan* p, const swp_group_state* st, void* const* slots, const swp_group_adjoint* adj,
                        const swp_flags* f, int t0, int nsteps, cudaStream_t s) {
  // slot 0 <- checkpoint (outside the graph: its source changes per window)
  size_t es = sizeof(typename cplx<T>::type);
  for (int g = 0; g < p->ng; ++g) {
    size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
    int rc = cuda_check(p, cudaMemcpyAsync(slots[g], st[g].fourier, bytes, cudaMemcpyDeviceToDevice, s), "window restore");
    if (rc) return rc;
  }
  auto body = [&](cudaStream_t cs) -> int {
    int rc = forward_steps<T>(p, st, f, t0, nsteps, 0, 0, slots, cs);
    if (rc) return rc;
    std::vector<swp_group_state> a(p->ng), b(p->ng);
    for (int k = nsteps - 1; k >= 0; --k) {
      for (int g = 0; g < p->ng; ++g) {
        size_t ss = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
        a[g] = st[g]; b[g] = st[g];
        a[g].fourier = (char*)slots[g] + (size_t)k * ss;
        b[g].fourier = (char*)slots[g] + (size_t)(k + 1) * ss;
      }
      rc = adjoint_step_impl<T>(p, a.data(), b.data(), adj, f, t0 + k, cs, false, true, k != nsteps - 1);
      if (rc) return rc;
    }
    return SWP_OK;
  };
  // the window map does not depend on t0 except through the RA-filtered carry,
  // which the adjoint never reads, so one graph serves every window of a length
  // (whether the window starts at t_start decides the projected first step)
  std::vector<uint64_t> key = {2, (uint64_t)nsteps, (uint64_t)(t0 == f->t_start)};
  key_flags(key, f);
  for (int g = 0; g < p->ng; ++g) {
    key.push_back((uint64_t)slots[g]); key.push_back((uint64_t)adj[g].lam); key.push_back((uint64_t)adj[g].lam_y);
    key.push_back((uint64_t)adj[g].grad); key.push_back((uint64_t)st[g].params); key.push_back((uint64_t)st[g].resid);
    key.push_back((uint64_t)st[g].member);
  }
  return run_graph(p, key, body, s);
}

template <typename T>
int time_kernels_impl(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, const swp_flags* f,
                      int nrep, float* ms, cudaStream_t s) {
  int nbs = 0, nbg = 0;
  SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LS.mode = 0;
  LG.mode = GM_STEP;
  StepCfg cfg = make_cfg(f);
  cfg.ra_mode = f->modalflag ? 2 : 1;
  cfg.diagnostics = 0;
  cfg.incremental = step_incremental(p, f, f->t_start + 1) ? 1 : 0;  // the steady-state step form
  LS.cfg = cfg;
  LG.cfg = cfg;
  GridLaunch<T> LGa = LG;
  SpecLaunch<T> LSa = LS;
  LGa.mode = GM_ADJ_STEP;
  LGa.cfg.lam_fg_tied = (f->forcflag && f->test == 0 && f->scheme == 0) ? 1 : 0;  // as inside an adjoint sweep
  // the steady state of a modified-Euler sweep: lambda of U, V, prev, mid already zero
  LGa.cfg.adj_zeroed = LSa.cfg.adj_zeroed = f->scheme == 0 ? 1 : 0;
  if (adj) {
    for (int g = 0; g < p->ng; ++g) {
      LGa.grp[g].primal = LG.grp[g].four;
      LGa.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
      LGa.grp[g].lamy = (typename cplx<T>::type*)adj[g].lam_y;
      LGa.grp[g].grad = adj[g].grad;
      LGa.grp[g].member = nullptr;
      LSa.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
      LSa.grp[g].lamY = (const typename cplx<T>::type*)adj[g].lam_y;
      LSa.grp[g].grad = adj[g].grad;
    }
  }
  int rc = update_coefs<T>(p, st, s);
  if (rc) return rc;
  cudaEvent_t ev[5];
  for (int i = 0; i < 5; ++i) cudaEventCreate(&ev[i]);
  double acc[4] = {0, 0, 0, 0};
  for (int r = 0; r < nrep; ++r) {
    cudaError_t le[4] = {cudaSuccess, cudaSuccess, cudaSuccess, cudaSuccess};
    cudaEventRecord(ev[0], s);
    le[0] = launch_step_spec<T>(p, LS, nbs, s);
    cudaEventRecord(ev[1], s);
    le[1] = launch_grid<T>(LG, nbg, p->grid_smem[GM_STEP], s);
    cudaEventRecord(ev[2], s);
    if (adj) {
      le[2] = launch_grid<T>(LGa, nbg, p->grid_smem[GM_ADJ_STEP], s);
      cudaEventRecord(ev[3], s);
      le[3] = launch_step_spec_adj<T>(p, LSa, nbs, s);
      cudaEventRecord(ev[4], s);
    }
    for (int k = 0; k < 4; ++k)
      if (le[k] != cudaSuccess) {
        for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
        return cuda_check(p, le[k], "timed kernel launch");
      }
    cudaError_t e = cudaEventSynchronize(adj ? ev[4] : ev[2]);
    if (e != cudaSuccess) { for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]); return cuda_check(p, e, "timed kernels"); }
    float t;
    cudaEventElapsedTime(&t, ev[0], ev[1]); acc[0] += t;
    cudaEventElapsedTime(&t, ev[1], ev[2]); acc[1] += t;
    if (adj) {
      cudaEventElapsedTime(&t, ev[2], ev[3]); acc[2] += t;
      cudaEventElapsedTime(&t, ev[3], ev[4]); acc[3] += t;
    }
  }
  for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  for (int k = 0; k < 4; ++k) ms[k] = nrep > 0 ? (float)(acc[k] / nrep) : 0.f;
  return cuda_check(p, cudaGetLastError(), "timed kernels");
}

template <typename T>
int forward_ckpt_impl(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps, int K,
                      void* const* ckpt, cudaStream_t s) {
  size_t es = sizeof(typename cplx<T>::type);
  auto body = [&](cudaStream_t cs) -> int {
    int nwin = (nsteps + K - 1) / K;
    for (int w = 0; w < nwin; ++w) {
      for (int g = 0; g < p->ng; ++g) {
        if (!active(p, g)) continue;
        size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
        int rc = cuda_check(p, cudaMemcpyAsync((char*)ckpt[g] + (size_t)w * bytes, st[g].fourier, bytes,
                                               cudaMemcpyDeviceToDevice, cs), "checkpoint copy");
        if (rc) return rc;
      }
      int n = std::min(K, nsteps - w * K);
      int rc = forward_steps<T>(p, st, f, t0 + w * K, n, 0, w == nwin - 1, nullptr, cs);
      if (rc) return rc;
    }
    return SWP_OK;
  };
  std::vector<uint64_t> key = {3, (uint64_t)t0, (uint64_t)nsteps, (uint64_t)K};
  key_flags(key, f);
  key_state(key, p, st);
  for (int g = 0; g < p->ng; ++g) key.push_back((uint64_t)ckpt[g]);
  return run_graph(p, key, body, s);
}

// Forward over [t0, t0+nsteps) keeping every state: states[g] holds nsteps+1
// contiguous Fourier states (slot 0 = the state at t0).  The final state is
// copied back into st[g].fourier.
template <typename T>
int forward_stored_impl(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps,
                        void* const* states, cudaStream_t s) {
  size_t es = sizeof(typename cplx<T>::type);
  auto body = [&](cudaStream_t cs) -> int {
    for (int g = 0; g < p->ng; ++g) {
      size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
      if (!active(p, g)) continue;
      int rc = cuda_check(p, cudaMemcpyAsync(states[g], st[g].fourier, bytes, cudaMemcpyDeviceToDevice, cs),
                          "stored forward: first state");
      if (rc) return rc;
    }
    int rc = forward_steps<T>(p, st, f, t0, nsteps, 0, 1, states, cs);
    if (rc) return rc;
    for (int g = 0; g < p->ng; ++g) {
      size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
      if (!active(p, g)) continue;
      rc = cuda_check(p, cudaMemcpyAsync(st[g].fourier, (const char*)states[g] + (size_t)nsteps * bytes, bytes,
                                         cudaMemcpyDeviceToDevice, cs), "stored forward: last state");
      if (rc) return rc;
    }
    return SWP_OK;
  };
  std::vector<uint64_t> key = {4, (uint64_t)t0, (uint64_t)nsteps};
  key_flags(key, f);
  key_state(key, p, st);
  for (int g = 0; g < p->ng; ++g) key.push_back((uint64_t)states[g]);
  return run_graph(p, key, body, s);
}

// Adjoint sweep over states stored by forward_stored_impl: steps t0+nsteps-1
// down to t0, no recomputation.
template <typename T>
int adjoint_stored_impl(swp_plan* p, const swp_group_state* st, void* const* states, const swp_group_adjoint* adj,
                        const swp_flags* f, int t0, int nsteps, cudaStream_t s) {
  size_t es = sizeof(typename cplx<T>::type);
  auto body = [&](cudaStream_t cs) -> int {
    int rc = update_coefs<T>(p, st, cs);
    if (rc) return rc;
    std::vector<swp_group_state> a(p->ng), b(p->ng);
    for (int k = nsteps - 1; k >= 0; --k) {
      for (int g = 0; g < p->ng; ++g) {
        size_t ss = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
        a[g] = st[g]; b[g] = st[g];
        a[g].fourier = (char*)states[g] + (size_t)k * ss;
        b[g].fourier = (char*)states[g] + (size_t)(k + 1) * ss;
      }
      rc = adjoint_step_impl<T>(p, a.data(), b.data(), adj, f, t0 + k, cs, false, true, k != nsteps - 1);
      if (rc) return rc;
    }
    return SWP_OK;
  };
  std::vector<uint64_t> key = {5, (uint64_t)t0, (uint64_t)nsteps};
  key_flags(key, f);
  for (int g = 0; g < p->ng; ++g) {
    key.push_back((uint64_t)states[g]); key.push_back((uint64_t)adj[g].lam); key.push_back((uint64_t)adj[g].lam_y);
    key.push_back((uint64_t)adj[g].grad); key.push_back((uint64_t)st[g].params); key.push_back((uint64_t)st[g].resid);
    key.push_back((uint64_t)st[g].member);
  }
  return run_graph(p, key, body, s);
}

// Shared memory of the SIMT Legendre kernels for the plan's current member tiles.
void refresh_spec_smem(swp_plan* p) {
  p->spec_smem = 0;
  p->spec_adj_smem = 0;
  const bool f64 = p->precision == SWP_FP64;
  for (int g = 0; g < p->ng; ++g) {
    const int J = p->geom[g].J;
    size_t ss = f64 ? spec_smem_bytes<double>(p->M[g], J, p->MT[g]) : spec_smem_bytes<float>(p->M[g], J, p->MT[g]);
    size_t sa = f64 ? spec_adj_smem_bytes<double>(p->M[g], J, p->MT[g]) : spec_adj_smem_bytes<float>(p->M[g], J, p->MT[g]);
    p->spec_smem = std::max(p->spec_smem, ss);
    p->spec_adj_smem = std::max(p->spec_adj_smem, sa);
  }
}

void clear_graphs(swp_plan* p) {
  for (auto& ge : p->graphs)
    if (ge.exec) cudaGraphExecDestroy(ge.exec);
  p->graphs.clear();
}

// Member tile (MT) of the SIMT Legendre kernels, per group: every power of two
// up to 8 (and B) whose kernels fit in shared memory is timed on the caller's
// buffers (forward Legendre kernel + its adjoint, steady-state step form), and
// the fastest is kept.  The tensor-core kernels use a fixed tile of 8.
template <typename T>
int autotune_impl(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, const swp_flags* f, int nrep,
                  int* chosen, cudaStream_t s) {
  const bool f64 = p->precision == SWP_FP64;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return fail(p, SWP_ERR_CUDA, "autotune events");
  int rc = update_coefs<T>(p, st, s);
  for (int g = 0; g < p->ng && rc == SWP_OK; ++g) {
    const int J = p->geom[g].J;
    const int keep = p->MT[g];
    const bool keep_tc = p->tc[g];
    // candidates: the tensor-core kernels (0, where the plan packed their basis)
    // and the SIMT member tiles 1, 2, 4, 8
    const bool tc_able = p->tcbasis[g] != nullptr;
    int best = keep, best_mt = keep;
    float best_ms = 3.4e38f;
    for (int mt = tc_able ? 0 : 1; mt <= 8 && mt <= std::max(1, p->B[g]); mt = mt ? 2 * mt : 1) {
      if (mt > 0) {
        size_t ss = f64 ? spec_smem_bytes<double>(p->M[g], J, mt) : spec_smem_bytes<float>(p->M[g], J, mt);
        size_t sa = f64 ? spec_adj_smem_bytes<double>(p->M[g], J, mt) : spec_adj_smem_bytes<float>(p->M[g], J, mt);
        if (ss > (size_t)SPEC_DYN_SMEM_MAX || sa > (size_t)SPEC_DYN_SMEM_MAX) continue;
        p->MT[g] = mt;
      }
      p->tc[g] = mt == 0;
      p->use_tc = false;
      for (int q = 0; q < p->ng; ++q) p->use_tc = p->use_tc || p->tc[q];
      refresh_spec_smem(p);
      int nbs = 0;
      SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
      LS.mode = 0;
      LS.cfg = make_cfg(f);
      LS.cfg.diagnostics = 0;
      LS.cfg.ra_mode = f->modalflag ? 2 : 1;
      LS.cfg.incremental = step_incremental(p, f, f->t_start + 1) ? 1 : 0;
      SpecLaunch<T> LA = LS;
      for (int q = 0; q < p->ng; ++q) {
        LA.grp[q].lam = (typename cplx<T>::type*)adj[q].lam;
        LA.grp[q].lamY = (const typename cplx<T>::type*)adj[q].lam_y;
        LA.grp[q].grad = adj[q].grad;
      }
      cudaError_t e = cudaSuccess;
      for (int r = 0; r < nrep + 1 && e == cudaSuccess; ++r) {  // the first repetition warms up
        if (r == 1) cudaEventRecord(e0, s);
        e = launch_step_spec<T>(p, LS, nbs, s);
        if (e == cudaSuccess) e = launch_step_spec_adj<T>(p, LA, nbs, s);
      }
      cudaEventRecord(e1, s);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) { rc = cuda_check(p, e, "autotune launch"); break; }
      if (ms < best_ms) {
        best_ms = ms;
        best = mt;
        if (mt > 0) best_mt = mt;
      }
    }
    // the SIMT tile stays set for the kernels without a tensor-core form
    // (tangent, explicit and semi-implicit steps)
    p->tc[g] = rc == SWP_OK ? best == 0 : keep_tc;
    p->MT[g] = rc == SWP_OK ? (best > 0 ? best : (best_mt > 0 ? best_mt : keep)) : keep;
    if (chosen) chosen[g] = p->tc[g] ? 0 : p->MT[g];
  }
  p->use_tc = false;
  for (int q = 0; q < p->ng; ++q) p->use_tc = p->use_tc || p->tc[q];
  refresh_spec_smem(p);
  clear_graphs(p);  // captured graphs hold the old launch shapes
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

}  // namespace

namespace swp {
// Entry points for other translation units (static_scratch.cu).
// The kernels move Fourier rows with 16-byte accesses (two latitudes in FP32,
// one in FP64), so every complex buffer must start on a 16-byte boundary, as
// cudaMalloc and torch allocations do.  A misaligned buffer is refused here
// rather than faulting on the device.
static bool misaligned(const void* q) { return q && ((uintptr_t)q & 15u) != 0; }
static int check_align(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj = nullptr,
                       void* const* arrays = nullptr, const swp_group_tangent* tan = nullptr) {
  for (int g = 0; g < p->ng; ++g) {
    if ((st && misaligned(st[g].fourier)) || (adj && (misaligned(adj[g].lam) || misaligned(adj[g].lam_y))) ||
        (arrays && misaligned(arrays[g])) || (tan && misaligned(tan[g].fourier)))
      return fail(p, SWP_ERR_ARG, "complex (Fourier) buffers must be 16-byte aligned");
  }
  return SWP_OK;
}

// Scheme switches every stepping entry checks (model.py:1531-1537).  The
// adjoint covers the three schemes with the classic filter (the semi-implicit
// scheme's adjoint propagates the state only: its parameter gradients are
// tangent runs).
int check_scheme(swp_plan* p, const swp_flags* f, bool adjoint) {
  if (f->scheme < 0 || f->scheme > 2) return fail(p, SWP_ERR_ARG, "scheme must be 0, 1 or 2");
  if (f->test < 0 || f->test > 2) return fail(p, SWP_ERR_ARG, "test must be 0 (None), 1 or 2");
  if (f->raw_filter && f->scheme == 1)
    return fail(p, SWP_ERR_ARG, "raw_filter is incompatible with the explicit scheme");
  if (adjoint && f->raw_filter)
    return fail(p, SWP_ERR_UNSUPPORTED,
                "the adjoint is implemented for the classic Robert-Asselin filter (RAW-filtered runs "
                "have tangents only)");
  return SWP_OK;
}

// Argument checks of the adjoint step, shared by swp_adjoint_step and its
// allocation-free variant (need_lamy = false: the variant supplies lam_y).
int adjoint_step_checks(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                        const swp_group_adjoint* adj, const swp_flags* f, bool need_lamy) {
  if (!p || !st_in || !st_out || !adj || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (int rc = check_scheme(p, f, true)) return rc;
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint of test=1 (fixed winds) is not implemented");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint runs with diagnostics off (no blow-up gate)");
  for (int g = 0; g < p->ng; ++g)
    if (!adj[g].lam || (need_lamy && !adj[g].lam_y) || !st_in[g].fourier || !st_out[g].fourier)
      return fail(p, SWP_ERR_ARG, "missing adjoint buffer");
  if (int rc = check_align(p, st_in, adj)) return rc;
  return check_align(p, st_out);
}

int adjoint_step_dispatch(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                          const swp_group_adjoint* adj, const swp_flags* f, int t, cudaStream_t s) {
  if (int rc = adjoint_step_checks(p, st_in, st_out, adj, f, true)) return rc;
  return p->precision == SWP_FP64 ? adjoint_step_impl<double>(p, st_in, st_out, adj, f, t, s)
                                  : adjoint_step_impl<float>(p, st_in, st_out, adj, f, t, s);
}
int plan_groups(const swp_plan* p) { return p->ng; }
size_t plan_lamy_bytes(const swp_plan* p, int g) {
  size_t es = p->precision == SWP_FP64 ? 16 : 8;
  return (size_t)5 * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
}
int plan_fail(swp_plan* p, int code, const char* msg) { return fail(p, code, msg); }
}  // namespace swp

extern "C" {

int swp_plan_create(int ngroups, const int* M, const int* B, int precision, swp_plan** out) {
  if (!out) return SWP_ERR_ARG;
  *out = nullptr;
  if (ngroups < 1 || ngroups > MAXG || !M || !B) return SWP_ERR_ARG;
  if (precision != SWP_FP64 && precision != SWP_FAST) return SWP_ERR_ARG;
  swp_plan* p = new (std::nothrow) swp_plan();
  if (!p) return SWP_ERR_ARG;
  p->precision = precision;
  p->ng = ngroups;
  const char* ng_env = getenv("SWP_NO_GRAPH");
  p->graphs_enabled = !(ng_env && ng_env[0] == '1');
  spec_set_attributes();
  grid_set_attributes();
  spec_tc_set_attributes();
  cudaStream_t s = 0;
  if (cudaMalloc(&p->d_sched, (MAXG + 1) * sizeof(SchedCounter)) != cudaSuccess ||
      cudaMemset(p->d_sched, 0, (MAXG + 1) * sizeof(SchedCounter)) != cudaSuccess) {
    p->err = "scheduler counter allocation failed";
    *out = p;
    return SWP_ERR_CUDA;
  }
  if (cudaMalloc(&p->d_err, sizeof(int)) != cudaSuccess || cudaMemset(p->d_err, 0, sizeof(int)) != cudaSuccess) {
    p->err = "device error word allocation failed";
    *out = p;
    return SWP_ERR_CUDA;
  }
  for (int g = 0; g < ngroups; ++g) {
    if (B[g] < 1) { p->err = "B must be >= 1"; *out = p; return SWP_ERR_ARG; }
    int rc = geometry_build(p->geom[g], M[g], s, p->err);
    if (rc != SWP_OK) { *out = p; return rc; }
    p->M[g] = M[g];
    p->B[g] = B[g];
    int J = p->geom[g].J, I = p->geom[g].I;
    bool f64 = precision == SWP_FP64;
    size_t cbytes = f64 ? CoefTables<double>::count(M[g], B[g], J) * sizeof(double)
                        : CoefTables<float>::count(M[g], B[g], J) * sizeof(float);
    if (cudaMalloc(&p->coefmem[g], cbytes) != cudaSuccess) {
      p->err = "coefficient table allocation failed";
      *out = p;
      return SWP_ERR_CUDA;
    }
    size_t cap = f64 ? 150 * 1024 : 110 * 1024;
    int mt = 8;
    while (mt > 1 && (f64 ? spec_smem_bytes<double>(M[g], J, mt) : spec_smem_bytes<float>(M[g], J, mt)) > cap) mt /= 2;
    p->MT[g] = std::min(mt, B[g]);
    // rows per grid CTA: fixed per truncation and mode at compile time (grid.cu grid_jb)
    p->JB[g] = grid_rows_per_cta(M[g], f64, GM_STEP);
    size_t ss = f64 ? spec_smem_bytes<double>(M[g], J, p->MT[g]) : spec_smem_bytes<float>(M[g], J, p->MT[g]);
    p->spec_smem = std::max(p->spec_smem, ss);
    size_t sa = f64 ? spec_adj_smem_bytes<double>(M[g], J, p->MT[g]) : spec_adj_smem_bytes<float>(M[g], J, p->MT[g]);
    p->spec_adj_smem = std::max(p->spec_adj_smem, sa);
    for (int mode = 0; mode < NGRIDMODE; ++mode) {
      const int jbm = grid_rows_per_cta(M[g], f64, mode);
      size_t gs = f64 ? grid_smem_bytes<double>(M[g], J, I, jbm, mode) : grid_smem_bytes<float>(M[g], J, I, jbm, mode);
      p->grid_smem[mode] = std::max(p->grid_smem[mode], gs);
    }
  }
  // tensor-core step kernels: every group of an FP32 plan, unless SWP_NO_TC=1
  const char* tc_env = getenv("SWP_NO_TC");
  const bool tc_on = precision == SWP_FAST && !(tc_env && tc_env[0] == '1');
  bool tc = false;
  for (int g = 0; g < ngroups; ++g) {
    p->tc[g] = tc_on && spec_tc_supported(M[g]);
    tc = tc || p->tc[g];
  }
  if (tc) {
    for (int g = 0; g < ngroups; ++g) {
      if (!p->tc[g]) continue;
      const bool adj = spec_tc_adj_supported(M[g]);
      if (cudaMalloc(&p->tcbasis[g], spec_tc_basis_floats(M[g]) * sizeof(float)) != cudaSuccess ||
          pack_tc_basis(p->geom[g], p->tcbasis[g], s) != SWP_OK ||
          (adj && cudaMalloc(&p->tcbasis_adj[g], spec_tc_adj_basis_floats(M[g]) * sizeof(float)) != cudaSuccess) ||
          (adj && pack_tc_basis_adj(p->geom[g], p->tcbasis_adj[g], s) != SWP_OK)) {
        p->err = "tensor-core basis packing failed";
        *out = p;
        return SWP_ERR_CUDA;
      }
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      p->err = "tensor-core basis packing failed";
      *out = p;
      return SWP_ERR_CUDA;
    }
    p->use_tc = true;
  }
  *out = p;
  return SWP_OK;
}

int swp_plan_destroy(swp_plan* p) {
  if (!p) return SWP_OK;
  for (auto& ge : p->graphs)
    if (ge.exec) cudaGraphExecDestroy(ge.exec);
  p->graphs.clear();
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->ev_fork) cudaEventDestroy(p->ev_fork);
  for (int g = 0; g < MAXG; ++g) {
    if (p->side[g]) cudaStreamDestroy(p->side[g]);
    if (p->ev_join[g]) cudaEventDestroy(p->ev_join[g]);
  }
  for (int g = 0; g < p->ng; ++g) {
    if (p->geom[g].mem) cudaFree(p->geom[g].mem);
    if (p->tcbasis[g]) cudaFree(p->tcbasis[g]);
    if (p->tcbasis_adj[g]) cudaFree(p->tcbasis_adj[g]);
    if (p->coefmem[g]) cudaFree(p->coefmem[g]);
  }
  if (p->d_err) cudaFree(p->d_err);
  if (p->d_sched) cudaFree(p->d_sched);
  delete p;
  return SWP_OK;
}

int swp_device_status(swp_plan* p, int* status, void* stream) {
  if (!p || !status) return SWP_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemsetAsync(p->d_err, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_check(p, e, "device status");
  *status = h;
  return SWP_OK;
}

int swp_plan_uses_tensor_cores(const swp_plan* p) {
  int mask = 0;
  if (p)
    for (int g = 0; g < p->ng; ++g) mask |= p->tc[g] ? (1 << g) : 0;
  return mask;
}

int swp_plan_dims(const swp_plan* p, int g, int* M, int* J, int* I, int* B) {
  if (!p || g < 0 || g >= p->ng) return SWP_ERR_ARG;
  if (M) *M = p->M[g];
  if (J) *J = p->geom[g].J;
  if (I) *I = p->geom[g].I;
  if (B) *B = p->B[g];
  return SWP_OK;
}

const char* swp_last_error(const swp_plan* p) { return p ? p->err.c_str() : "null plan"; }

int swp_geometry(const swp_plan* p, int g, double* mus, double* w, double* Pmn, double* Hmn, void* stream) {
  if (!p || g < 0 || g >= p->ng) return SWP_ERR_ARG;
  swp_plan* q = const_cast<swp_plan*>(p);
  cudaStream_t s = (cudaStream_t)stream;
  const GroupGeom& gg = p->geom[g];
  if (mus) { int rc = cuda_check(q, cudaMemcpyAsync(mus, gg.mu, gg.J * 8, cudaMemcpyDeviceToDevice, s), "mus copy"); if (rc) return rc; }
  if (w) { int rc = cuda_check(q, cudaMemcpyAsync(w, gg.w, gg.J * 8, cudaMemcpyDeviceToDevice, s), "w copy"); if (rc) return rc; }
  if (Pmn && Hmn) {
    if (geometry_dense(gg, Pmn, Hmn, s) != SWP_OK) return fail(q, SWP_ERR_CUDA, "dense basis kernel");
  } else if (Pmn || Hmn) {
    return fail(q, SWP_ERR_ARG, "Pmn and Hmn must be requested together");
  }
  return SWP_OK;
}

int swp_init_state(swp_plan* p, const swp_group_state* st, void* const* phys_ic, const swp_flags* f, void* stream) {
  if (!p || !st || !phys_ic || !f) return fail(p, SWP_ERR_ARG, "null argument");
  for (int g = 0; g < p->ng; ++g)
    if (!st[g].fourier || !st[g].resid || !st[g].params || !st[g].member || !phys_ic[g])
      return fail(p, SWP_ERR_ARG, "missing state buffer");
  if (f->diagnostics)
    for (int g = 0; g < p->ng; ++g)
      if (!st[g].diag) return fail(p, SWP_ERR_ARG, "diagnostics requested without a diag buffer");
  if (int rc = check_align(p, st)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? init_impl<double>(p, st, phys_ic, f, s) : init_impl<float>(p, st, phys_ic, f, s);
}

int swp_diagnose_winds(swp_plan* p, const swp_group_state* st, void* const* ed, void* const* uv, void* stream) {
  if (!p || !st || !ed || !uv) return fail(p, SWP_ERR_ARG, "null argument");
  if (int rc = check_align(p, st)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? winds_impl<double>(p, st, ed, uv, s) : winds_impl<float>(p, st, ed, uv, s);
}

int swp_forward(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps, int row0,
                int write_prev_last, void* stream) {
  if (!p || !st || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (nsteps < 0) return fail(p, SWP_ERR_ARG, "nsteps must be >= 0");
  if (int rc = check_scheme(p, f, false)) return rc;
  for (int g = 0; g < p->ng; ++g) {
    if (!st[g].fourier || !st[g].params || !st[g].member) return fail(p, SWP_ERR_ARG, "missing state buffer");
    if (f->diagnostics && !st[g].diag) return fail(p, SWP_ERR_ARG, "diagnostics requested without a diag buffer");
  }
  if (int rc = check_align(p, st)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? forward_impl<double>(p, st, f, t0, nsteps, row0, write_prev_last, s)
                                  : forward_impl<float>(p, st, f, t0, nsteps, row0, write_prev_last, s);
}

static int check_tangent(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, const swp_flags* f) {
  if (!p || !st || !tan || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (int rc = check_scheme(p, f, false)) return rc;
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "tangent of test=1 (fixed winds) is not implemented");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "tangent runs with diagnostics off (no blow-up gate)");
  for (int g = 0; g < p->ng; ++g)
    if (!tan[g].fourier || !tan[g].resid || !tan[g].dparams || !tan[g].dweights || !st[g].fourier ||
        !st[g].params || !st[g].member)
      return fail(p, SWP_ERR_ARG, "missing tangent buffer");
  return check_align(p, st, nullptr, nullptr, tan);
}

int swp_tangent_init(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, void* const* phys,
                     void* const* dphys, const swp_flags* f, void* stream) {
  if (int rc = check_tangent(p, st, tan, f)) return rc;
  if (!phys || !dphys) return fail(p, SWP_ERR_ARG, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? tangent_init_impl<double>(p, st, tan, phys, dphys, f, s)
                                  : tangent_init_impl<float>(p, st, tan, phys, dphys, f, s);
}

int swp_tangent_forward(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, const swp_flags* f,
                        int t0, int nsteps, void* stream) {
  if (int rc = check_tangent(p, st, tan, f)) return rc;
  if (nsteps < 0) return fail(p, SWP_ERR_ARG, "nsteps must be >= 0");
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? tangent_forward_impl<double>(p, st, tan, f, t0, nsteps, s)
                                  : tangent_forward_impl<float>(p, st, tan, f, t0, nsteps, s);
}

int swp_tangent_output(swp_plan* p, const swp_group_state* st, const swp_group_tangent* tan, void* const* out,
                       const swp_flags* f, void* stream) {
  if (int rc = check_tangent(p, st, tan, f)) return rc;
  if (!out) return fail(p, SWP_ERR_ARG, "null argument");
  swp_group_state tst[MAXG];
  tangent_states(p, st, tan, tst);
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? output_impl<double>(p, tst, out, f, s, st, tan)
                                  : output_impl<float>(p, tst, out, f, s, st, tan);
}

int swp_output_physical(swp_plan* p, const swp_group_state* st, void* const* out, const swp_flags* f, void* stream) {
  if (!p || !st || !out || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (int rc = check_align(p, st)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? output_impl<double>(p, st, out, f, s) : output_impl<float>(p, st, out, f, s);
}

int swp_state_copy(swp_plan* p, const swp_group_state* st, void* const* ckpt, int dir, void* stream) {
  if (!p || !st || !ckpt) return fail(p, SWP_ERR_ARG, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  size_t es = p->precision == SWP_FP64 ? 16 : 8;
  for (int g = 0; g < p->ng; ++g) {
    size_t bytes = (size_t)SWP_NFOURIER * (p->M[g] + 1) * p->B[g] * p->geom[g].J * es;
    void* dst = dir == 0 ? ckpt[g] : st[g].fourier;
    const void* src = dir == 0 ? st[g].fourier : ckpt[g];
    int rc = cuda_check(p, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s), "state copy");
    if (rc) return rc;
  }
  return SWP_OK;
}

int swp_adjoint_step(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                     const swp_group_adjoint* adj, const swp_flags* f, int t, void* stream) {
  if (int rc = adjoint_step_checks(p, st_in, st_out, adj, f, true)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_step_impl<double>(p, st_in, st_out, adj, f, t, s)
                                  : adjoint_step_impl<float>(p, st_in, st_out, adj, f, t, s);
}

int swp_adjoint_seed(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, void* const* dphys, void* stream) {
  if (!p || !st || !adj || !dphys) return fail(p, SWP_ERR_ARG, "null argument");
  if (int rc = check_align(p, st, adj)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_seed_impl<double>(p, st, adj, dphys, s)
                                  : adjoint_seed_impl<float>(p, st, adj, dphys, s);
}

int swp_adjoint_init(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, void* const* phys_ic,
                     void* const* dic, const swp_flags* f, void* stream) {
  if (!p || !st || !adj || !phys_ic || !dic || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint of test=1 (fixed winds) is not implemented");
  if (int rc = check_align(p, st, adj)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_init_impl<double>(p, st, adj, phys_ic, dic, f, s)
                                  : adjoint_init_impl<float>(p, st, adj, phys_ic, dic, f, s);
}

int swp_adjoint_window(swp_plan* p, const swp_group_state* st, void* const* slots, const swp_group_adjoint* adj,
                       const swp_flags* f, int t0, int nsteps, void* stream) {
  if (!p || !st || !slots || !adj || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (nsteps < 1) return fail(p, SWP_ERR_ARG, "nsteps must be >= 1");
  if (int rc = check_scheme(p, f, true)) return rc;
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint of test=1 (fixed winds) is not implemented");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint runs with diagnostics off (no blow-up gate)");
  for (int g = 0; g < p->ng; ++g)
    if (!slots[g] || !adj[g].lam || !adj[g].lam_y || !st[g].fourier) return fail(p, SWP_ERR_ARG, "missing buffer");
  if (int rc = check_align(p, st, adj, slots)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_window_impl<double>(p, st, slots, adj, f, t0, nsteps, s)
                                  : adjoint_window_impl<float>(p, st, slots, adj, f, t0, nsteps, s);
}

int swp_time_kernels(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, const swp_flags* f,
                     int nrep, float* ms_out, void* stream) {
  if (!p || !st || !f || !ms_out || nrep < 1) return fail(p, SWP_ERR_ARG, "bad argument");
  if (int rc = check_align(p, st, adj)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? time_kernels_impl<double>(p, st, adj, f, nrep, ms_out, s)
                                  : time_kernels_impl<float>(p, st, adj, f, nrep, ms_out, s);
}

int swp_forward_checkpointed(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps,
                             int ckpt_every, void* const* ckpt, void* stream) {
  if (!p || !st || !f || !ckpt) return fail(p, SWP_ERR_ARG, "null argument");
  if (nsteps < 1 || ckpt_every < 1) return fail(p, SWP_ERR_ARG, "nsteps and ckpt_every must be >= 1");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "checkpointed forward runs with diagnostics off");
  if (int rc = check_scheme(p, f, false)) return rc;
  for (int g = 0; g < p->ng; ++g)
    if (!ckpt[g] || !st[g].fourier || !st[g].params || !st[g].member) return fail(p, SWP_ERR_ARG, "missing buffer");
  if (int rc = check_align(p, st)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? forward_ckpt_impl<double>(p, st, f, t0, nsteps, ckpt_every, ckpt, s)
                                  : forward_ckpt_impl<float>(p, st, f, t0, nsteps, ckpt_every, ckpt, s);
}

int swp_forward_stored(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps,
                       void* const* states, void* stream) {
  if (!p || !st || !f || !states) return fail(p, SWP_ERR_ARG, "null argument");
  if (nsteps < 1) return fail(p, SWP_ERR_ARG, "nsteps must be >= 1");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "stored forward runs with diagnostics off");
  if (int rc = check_scheme(p, f, false)) return rc;
  for (int g = 0; g < p->ng; ++g)
    if (!states[g] || !st[g].fourier || !st[g].params || !st[g].member) return fail(p, SWP_ERR_ARG, "missing buffer");
  if (int rc = check_align(p, st, nullptr, states)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? forward_stored_impl<double>(p, st, f, t0, nsteps, states, s)
                                  : forward_stored_impl<float>(p, st, f, t0, nsteps, states, s);
}

int swp_adjoint_stored(swp_plan* p, const swp_group_state* st, void* const* states, const swp_group_adjoint* adj,
                       const swp_flags* f, int t0, int nsteps, void* stream) {
  if (!p || !st || !states || !adj || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (nsteps < 1) return fail(p, SWP_ERR_ARG, "nsteps must be >= 1");
  if (int rc = check_scheme(p, f, true)) return rc;
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint of test=1 (fixed winds) is not implemented");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint runs with diagnostics off (no blow-up gate)");
  for (int g = 0; g < p->ng; ++g)
    if (!states[g] || !adj[g].lam || !adj[g].lam_y || !st[g].params) return fail(p, SWP_ERR_ARG, "missing buffer");
  if (int rc = check_align(p, st, adj, states)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_stored_impl<double>(p, st, states, adj, f, t0, nsteps, s)
                                  : adjoint_stored_impl<float>(p, st, states, adj, f, t0, nsteps, s);
}

int swp_plan_autotune(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, const swp_flags* f,
                      int nrep, int* chosen_mt, void* stream) {
  if (!p || !st || !adj || !f || nrep < 1) return fail(p, SWP_ERR_ARG, "bad argument");
  for (int g = 0; g < p->ng; ++g)
    if (!st[g].fourier || !st[g].params || !st[g].member || !adj[g].lam || !adj[g].lam_y)
      return fail(p, SWP_ERR_ARG, "missing buffer");
  if (int rc = check_align(p, st, adj)) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? autotune_impl<double>(p, st, adj, f, nrep, chosen_mt, s)
                                  : autotune_impl<float>(p, st, adj, f, nrep, chosen_mt, s);
}

int swp_plan_tiles(const swp_plan* p, int g, int* mt, int* jb) {
  if (!p || g < 0 || g >= p->ng) return SWP_ERR_ARG;
  if (mt) *mt = p->MT[g];
  if (jb) *jb = p->JB[g];
  return SWP_OK;
}

int swp_plan_set_tile(swp_plan* p, int g, int mt) {
  if (!p || g < 0 || g >= p->ng) return SWP_ERR_ARG;
  const bool f64 = p->precision == SWP_FP64;
  const int J = p->geom[g].J;
  if (mt == 0) {  // the tensor-core kernels
    if (!p->tcbasis[g]) return fail(p, SWP_ERR_ARG, "this group cannot run the tensor-core kernels");
    if (!p->tc[g]) clear_graphs(p);
    p->tc[g] = true;
    p->use_tc = true;
    return SWP_OK;
  }
  if (mt < 1 || mt > 8 || (mt & (mt - 1)) != 0) return fail(p, SWP_ERR_ARG, "member tile must be 0, 1, 2, 4 or 8");
  size_t ss = f64 ? spec_smem_bytes<double>(p->M[g], J, mt) : spec_smem_bytes<float>(p->M[g], J, mt);
  size_t sa = f64 ? spec_adj_smem_bytes<double>(p->M[g], J, mt) : spec_adj_smem_bytes<float>(p->M[g], J, mt);
  if (ss > (size_t)SPEC_DYN_SMEM_MAX || sa > (size_t)SPEC_DYN_SMEM_MAX)
    return fail(p, SWP_ERR_ARG, "member tile does not fit in shared memory");
  p->MT[g] = mt;
  p->tc[g] = false;
  p->use_tc = false;
  for (int q = 0; q < p->ng; ++q) p->use_tc = p->use_tc || p->tc[q];
  refresh_spec_smem(p);
  clear_graphs(p);
  return SWP_OK;
}

int swp_plan_set_wait_limit(swp_plan* p, unsigned int max_polls) {
  if (!p) return SWP_ERR_ARG;
  if (p->tc_wait_limit != max_polls) clear_graphs(p);  // the limit is a launch argument of the captured kernels
  p->tc_wait_limit = max_polls;
  return SWP_OK;
}

int swp_plan_set_concurrency(swp_plan* p, int on) {
  if (!p) return fail(p, SWP_ERR_ARG, "null plan");
  if (p->concurrent != (on != 0)) clear_graphs(p);  // graphs are captured per schedule
  p->concurrent = on != 0;
  return SWP_OK;
}

}  // extern "C"
