// C ABI of libswampe_gb300: plan lifetime, launch decomposition and the
// step loop.  See include/swampe_gb300.h for the contract of each symbol.
#include <algorithm>
#include <cstring>
#include <new>
#include "swp_internal.h"

using namespace swp;

struct swp_plan {
  int precision = SWP_FP64;
  int ng = 0;
  GroupGeom geom[MAXG];
  int M[MAXG] = {}, B[MAXG] = {}, MT[MAXG] = {}, JB[MAXG] = {};
  size_t spec_smem = 0;
  size_t spec_adj_smem = 0;
  size_t grid_smem[8] = {};
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

template <typename T>
SpecLaunch<T> make_spec(const swp_plan* p, const swp_group_state* st, int& nblocks) {
  SpecLaunch<T> L;
  memset(&L, 0, sizeof(L));
  L.ng = p->ng;
  int acc = 0;
  for (int g = 0; g < p->ng; ++g) {
    SpecGroup<T>& G = L.grp[g];
    G.g = p->geom[g].view<T>();
    G.B = p->B[g];
    G.MT = p->MT[g];
    G.ntb = (G.B + G.MT - 1) / G.MT;
    G.four = (typename cplx<T>::type*)st[g].fourier;
    G.par = st[g].params;
    G.member = st[g].member;
    G.diag = st[g].diag;
    L.prefix[g] = acc;
    acc += (p->M[g] + 1) * G.ntb;
  }
  L.prefix[p->ng] = acc;
  nblocks = acc;
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
    G.B = p->B[g];
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
  c.forcflag = f->forcflag;
  c.diffflag = f->diffflag;
  c.test = f->test;
  c.diagnostics = f->diagnostics;
  c.blowup = f->blowup;
  return c;
}

template <typename T>
int forward_impl(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps,
                 int row0, int write_prev_last, cudaStream_t s) {
  int nbs = 0, nbg = 0;
  SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LS.mode = 0;
  LG.mode = GM_STEP;
  StepCfg cfg = make_cfg(f);
  for (int k = 0; k < nsteps; ++k) {
    int t = t0 + k;
    cfg.step = row0 + k;
    cfg.ra_mode = (f->modalflag && t > 2) ? 2 : 1;
    cfg.write_prev = (f->scheme == 1) || (write_prev_last && k == nsteps - 1);
    LS.cfg = cfg;
    LG.cfg = cfg;
    for (int g = 0; g < p->ng; ++g) {
      size_t PS = (size_t)p->B[g] * p->geom[g].J * p->geom[g].I;
      LG.grp[g].hist = st[g].hist ? (T*)st[g].hist + (size_t)(row0 + k) * 5 * PS : nullptr;
    }
    cudaError_t e = launch_spec<T>(LS, nbs, p->spec_smem, s);
    if (e != cudaSuccess) return cuda_check(p, e, "spectral kernel launch");
    e = launch_grid<T>(LG, nbg, p->grid_smem[GM_STEP], s);
    if (e != cudaSuccess) return cuda_check(p, e, "grid kernel launch");
  }
  return SWP_OK;
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
int output_impl(swp_plan* p, const swp_group_state* st, void* const* out, const swp_flags* f, cudaStream_t s) {
  int nbg = 0;
  GridLaunch<T> LG = make_grid<T>(p, st, nbg);
  LG.mode = GM_OUTPUT;
  LG.cfg = make_cfg(f);
  LG.cfg.diagnostics = 0;
  for (int g = 0; g < p->ng; ++g) LG.grp[g].phys_out = (T*)out[g];
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
  SpecLaunch<T> LS = make_spec<T>(p, st, nbs);
  LS.mode = 2;
  e = launch_spec<T>(LS, nbs, p->spec_smem, s);
  if (e != cudaSuccess) return cuda_check(p, e, "winds Legendre kernel");
  LG.mode = GM_WINDS;
  for (int g = 0; g < p->ng; ++g) { LG.grp[g].phys_out = (T*)uv[g]; LG.grp[g].member = nullptr; }
  e = launch_grid<T>(LG, nbg, p->grid_smem[GM_WINDS], s);
  return cuda_check(p, e, "winds inverse transform");
}

template <typename T>
int adjoint_step_impl(swp_plan* p, const swp_group_state* st_in, const swp_group_state* st_out,
                      const swp_group_adjoint* adj, const swp_flags* f, cudaStream_t s) {
  int nbg = 0, nbs = 0;
  GridLaunch<T> LG = make_grid<T>(p, st_out, nbg);
  LG.mode = GM_ADJ_STEP;
  LG.cfg = make_cfg(f);
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
  for (int g = 0; g < p->ng; ++g) {
    LS.grp[g].lam = (typename cplx<T>::type*)adj[g].lam;
    LS.grp[g].lamY = (const typename cplx<T>::type*)adj[g].lam_y;
    LS.grp[g].grad = adj[g].grad;
  }
  e = launch_spec_adj<T>(LS, nbs, p->spec_adj_smem, s);
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

}  // namespace

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
  cudaStream_t s = 0;
  for (int g = 0; g < ngroups; ++g) {
    if (B[g] < 1) { p->err = "B must be >= 1"; *out = p; return SWP_ERR_ARG; }
    int rc = geometry_build(p->geom[g], M[g], s, p->err);
    if (rc != SWP_OK) { *out = p; return rc; }
    p->M[g] = M[g];
    p->B[g] = B[g];
    int J = p->geom[g].J, I = p->geom[g].I;
    bool f64 = precision == SWP_FP64;
    size_t cap = f64 ? 150 * 1024 : 110 * 1024;
    int mt = 8;
    while (mt > 1 && (f64 ? spec_smem_bytes<double>(M[g], J, mt) : spec_smem_bytes<float>(M[g], J, mt)) > cap) mt /= 2;
    p->MT[g] = std::min(mt, B[g]);
    int jb = 8;
    size_t gcap = 100 * 1024;
    while (jb > 1 && ((J % jb) != 0 ||
                      (f64 ? grid_smem_bytes<double>(M[g], J, I, jb, GM_STEP) : grid_smem_bytes<float>(M[g], J, I, jb, GM_STEP)) > gcap))
      jb /= 2;
    p->JB[g] = jb;
    size_t ss = f64 ? spec_smem_bytes<double>(M[g], J, p->MT[g]) : spec_smem_bytes<float>(M[g], J, p->MT[g]);
    p->spec_smem = std::max(p->spec_smem, ss);
    size_t sa = f64 ? spec_adj_smem_bytes<double>(M[g], J, p->MT[g]) : spec_adj_smem_bytes<float>(M[g], J, p->MT[g]);
    p->spec_adj_smem = std::max(p->spec_adj_smem, sa);
    for (int mode = 0; mode < 8; ++mode) {
      size_t gs = f64 ? grid_smem_bytes<double>(M[g], J, I, jb, mode) : grid_smem_bytes<float>(M[g], J, I, jb, mode);
      p->grid_smem[mode] = std::max(p->grid_smem[mode], gs);
    }
  }
  *out = p;
  return SWP_OK;
}

int swp_plan_destroy(swp_plan* p) {
  if (!p) return SWP_OK;
  for (int g = 0; g < p->ng; ++g)
    if (p->geom[g].mem) cudaFree(p->geom[g].mem);
  delete p;
  return SWP_OK;
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
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? init_impl<double>(p, st, phys_ic, f, s) : init_impl<float>(p, st, phys_ic, f, s);
}

int swp_diagnose_winds(swp_plan* p, const swp_group_state* st, void* const* ed, void* const* uv, void* stream) {
  if (!p || !st || !ed || !uv) return fail(p, SWP_ERR_ARG, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? winds_impl<double>(p, st, ed, uv, s) : winds_impl<float>(p, st, ed, uv, s);
}

int swp_forward(swp_plan* p, const swp_group_state* st, const swp_flags* f, int t0, int nsteps, int row0,
                int write_prev_last, void* stream) {
  if (!p || !st || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (nsteps < 0) return fail(p, SWP_ERR_ARG, "nsteps must be >= 0");
  if (f->scheme != 0 && f->scheme != 1) return fail(p, SWP_ERR_ARG, "scheme must be 0 or 1");
  if (f->test < 0 || f->test > 2) return fail(p, SWP_ERR_ARG, "test must be 0 (None), 1 or 2");
  for (int g = 0; g < p->ng; ++g) {
    if (!st[g].fourier || !st[g].params || !st[g].member) return fail(p, SWP_ERR_ARG, "missing state buffer");
    if (f->diagnostics && !st[g].diag) return fail(p, SWP_ERR_ARG, "diagnostics requested without a diag buffer");
  }
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? forward_impl<double>(p, st, f, t0, nsteps, row0, write_prev_last, s)
                                  : forward_impl<float>(p, st, f, t0, nsteps, row0, write_prev_last, s);
}

int swp_output_physical(swp_plan* p, const swp_group_state* st, void* const* out, const swp_flags* f, void* stream) {
  if (!p || !st || !out || !f) return fail(p, SWP_ERR_ARG, "null argument");
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
  (void)t;  // the modified-Euler step map does not depend on t
  if (!p || !st_in || !st_out || !adj || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (f->scheme != 0) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint is implemented for the modified-Euler scheme");
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint of test=1 (fixed winds) is not implemented");
  if (f->diagnostics) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint runs with diagnostics off (no blow-up gate)");
  for (int g = 0; g < p->ng; ++g)
    if (!adj[g].lam || !adj[g].lam_y || !st_in[g].fourier || !st_out[g].fourier) return fail(p, SWP_ERR_ARG, "missing adjoint buffer");
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_step_impl<double>(p, st_in, st_out, adj, f, s)
                                  : adjoint_step_impl<float>(p, st_in, st_out, adj, f, s);
}

int swp_adjoint_seed(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, void* const* dphys, void* stream) {
  if (!p || !st || !adj || !dphys) return fail(p, SWP_ERR_ARG, "null argument");
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_seed_impl<double>(p, st, adj, dphys, s)
                                  : adjoint_seed_impl<float>(p, st, adj, dphys, s);
}

int swp_adjoint_init(swp_plan* p, const swp_group_state* st, const swp_group_adjoint* adj, void* const* phys_ic,
                     void* const* dic, const swp_flags* f, void* stream) {
  if (!p || !st || !adj || !phys_ic || !dic || !f) return fail(p, SWP_ERR_ARG, "null argument");
  if (f->test == 1) return fail(p, SWP_ERR_UNSUPPORTED, "adjoint of test=1 (fixed winds) is not implemented");
  cudaStream_t s = (cudaStream_t)stream;
  return p->precision == SWP_FP64 ? adjoint_init_impl<double>(p, st, adj, phys_ic, dic, f, s)
                                  : adjoint_init_impl<float>(p, st, adj, phys_ic, dic, f, s);
}

}  // extern "C"
