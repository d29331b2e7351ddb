// Internal host/device declarations shared by the translation units of
// libswampe_gb300.so.  Nothing here crosses the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>
#include "swp_common.cuh"
#include "../../include/swampe_gb300.h"

namespace swp {

enum BasisIndex { B_PW_F = 0, B_HW_F, B_P_F, B_H_F, B_P_I, B_H_I, B_PW_I, B_HW_I };

// Per-member scalars kept on the device: weights of the initial-condition
// residual in the physical curr / RA-prev fields, the blow-up flag and
// whether the member has taken a step.
enum MemberScalar { MS_WCURR = 0, MS_WMID, MS_DEAD, MS_UPDATED, NMEMBER };
// Per-step diagnostics: sum for the RMS wind (before sqrt), min wind speed,
// min/max of the RA-filtered Phi, blow-up flag.
enum DiagIndex { D_RMS2 = 0, D_SPIN, D_PHIMIN, D_PHIMAX, D_DEAD, NDIAG };
// Parameter gradients accumulated by the adjoint.
enum GradIndex { G_TAURAD = 0, G_TAUDRAG, G_DPHIEQ, G_PHIBAR, NGRAD };
// Parameter tangents of the tangent-linear model: the adjoint's four, then
// those that enter only the coefficient tables.
enum TangentIndex {
  T_TAURAD = 0, T_TAUDRAG, T_DPHIEQ, T_PHIBAR, T_A, T_DT, T_K6, T_K6PHI, T_OMEGA, T_SIALPHA, T_ALPHA, T_WALPHA,
  NTANGENT
};
static_assert(NTANGENT == SWP_NTANGENT, "tangent rows of the C ABI");

struct GroupGeom {
  int M = 0, J = 0, I = 0, L = 0;
  size_t nbasis = 0, bytes = 0;
  void* mem = nullptr;
  double *mu = nullptr, *w = nullptr, *onemu2 = nullptr, *area = nullptr;
  double *ihalf64 = nullptr, *coslat64 = nullptr;
  float *ihalf32 = nullptr, *coslat32 = nullptr;
  int* boff = nullptr;
  double* b64[8] = {};
  float* b32[8] = {};
  double2 *twL64 = nullptr, *twI64 = nullptr;
  float2 *twL32 = nullptr, *twI32 = nullptr;
  double* dayc64 = nullptr;
  float* dayc32 = nullptr;

  template <typename T> Geom<T> view() const;
};

template <> inline Geom<double> GroupGeom::view<double>() const {
  Geom<double> g;
  g.M = M; g.J = J; g.I = I; g.L = L;
  g.mu = mu; g.w = w; g.onemu2 = onemu2; g.area = area; g.boff = boff;
  g.Pw_f = b64[B_PW_F]; g.Hw_f = b64[B_HW_F]; g.P_f = b64[B_P_F]; g.H_f = b64[B_H_F];
  g.P_i = b64[B_P_I]; g.H_i = b64[B_H_I]; g.Pw_i = b64[B_PW_I]; g.Hw_i = b64[B_HW_I];
  g.twL = twL64; g.twI = twI64; g.dayc = dayc64;
  g.ihalf = ihalf64; g.coslat = coslat64;
  return g;
}
template <> inline Geom<float> GroupGeom::view<float>() const {
  Geom<float> g;
  g.M = M; g.J = J; g.I = I; g.L = L;
  g.mu = mu; g.w = w; g.onemu2 = onemu2; g.area = area; g.boff = boff;
  g.Pw_f = b32[B_PW_F]; g.Hw_f = b32[B_HW_F]; g.P_f = b32[B_P_F]; g.H_f = b32[B_H_F];
  g.P_i = b32[B_P_I]; g.H_i = b32[B_H_I]; g.Pw_i = b32[B_PW_I]; g.Hw_i = b32[B_HW_I];
  g.twL = twL32; g.twI = twI32; g.dayc = dayc32;
  g.ihalf = ihalf32; g.coslat = coslat32;
  return g;
}

int geometry_build(GroupGeom& gg, int M, cudaStream_t stream, std::string& err);
int geometry_dense(const GroupGeom& gg, double* Pd, double* Hd, cudaStream_t stream);

constexpr int MAXG = 4;

// Per-call coefficient tables (coefs.cu): every factor of a step that depends
// only on a member's parameters, and on n or the latitude, computed once per
// call in FP64 with the reference's expressions and stored in the compute
// type, so that the step kernels do no FP64 arithmetic of their own.
//   nco[q][b][n]   q: hyperdiffusion sigma, sigmaPhi, sigma - 1, sigmaPhi - 1
//                     (filters.py:95-151), a / (n(n+1)) (spectral_transform.py:577),
//                     the exponential sigma, sigmaPhi of the semi-implicit scheme
//                     (filters.py:154-213)
//   jco[b][j]      tstepcoeff = 2 dt / (a (1 - mu_j^2)) (time_stepping.py:491-500)
//   mco[q][b]      scalar factors of the tendencies (modEuler_tdiff.py, explicit_tdiff.py)
enum NCoef {
  NC_SIG = 0, NC_SIGP, NC_SIGM1, NC_SIGPM1, NC_TC, NC_SIGX, NC_SIGPX,
  NC_DSIG, NC_DSIGP, NC_DTC,  // tangents of sigma, sigmaPhi, a/(n(n+1)) (tangent-linear launches)
  NC_DSIGX, NC_DSIGPX,        // tangents of the exponential sigmas
  NNCO
};
enum MCoef {
  MC_DT = 0,   // dt
  MC_T2,       // (2 dt / a^2) / 4
  MC_IA2,      // 1 / a^2
  MC_HPB,      // Phibar / 2
  MC_DTPB,     // dt Phibar
  MC_PBA2,     // Phibar / a^2
  MC_PFD,      // (dt / 2) / a^2
  MC_2DTPB,    // 2 dt Phibar
  MC_2DT,      // 2 dt
  MC_ITD,      // 1 / taudrag
  MC_OM,       // omega / sqrt(0.375)  (the planetary-vorticity part of eta_{0,1})
  MC_ALPHA,    // Robert-Asselin alpha
  MC_SIXI,     // 2 dt si_alpha            (implicit share of the semi-implicit step)
  MC_SIEX,     // 2 dt (1 - si_alpha)      (explicit share)
  MC_SIITD,    // 1 / taudrag, 0 for the taudrag = -1 sentinel
  MC_SIITR,    // 1 / taurad
  MC_RAWM,     // alpha williams_alpha       (RAW: displacement of the mid level)
  MC_RAWN,     // alpha (1 - williams_alpha) (RAW: displacement of the new level)
  MC_PB,       // Phibar
  // tangents of the step factors along the call's parameter tangents (tangent-linear launches)
  MC_DT2, MC_DIA2, MC_DHPB, MC_DDTPB, MC_DPBA2, MC_DPFD, MC_DDT, MC_DOM,
  MC_DSIXI, MC_DSIEX, MC_DSIITD, MC_DSIITR,  // of the semi-implicit shares and rates
  MC_DITD,     // of 1 / taudrag (explicit scheme; no sentinel)
  MC_DALPHA, MC_DRAWM, MC_DRAWN,  // of alpha, alpha williams_alpha, alpha (1 - williams_alpha)
  NMCO
};
template <typename T>
struct CoefTables {
  T* nco = nullptr;   // [NNCO][B][M+1]
  T* jco = nullptr;   // [B][J]
  T* djco = nullptr;  // [B][J] tangent of tstepcoeff
  T* mco = nullptr;   // [NMCO][B]
  static size_t count(int M, int B, int J) {
    return (size_t)NNCO * B * (M + 1) + (size_t)2 * B * J + (size_t)NMCO * B;
  }
  void carve(T* base, int M, int B, int J) {
    nco = base;
    jco = nco + (size_t)NNCO * B * (M + 1);
    djco = jco + (size_t)B * J;
    mco = djco + (size_t)B * J;
  }
};
// dpar: [NTANGENT][B] parameter tangents, or null (the tangent rows are then zero)
template <typename T>
cudaError_t launch_coefs(const double* par, const double* onemu2, int M, int B, int J, const CoefTables<T>& C,
                         cudaStream_t s, const double* dpar = nullptr);

// --------------------------------------------------------------- spectral ---
template <typename T>
struct SpecGroup {
  Geom<T> g;
  int B, MT, ntb;                       // members, members per tile, tiles along b
  typename cplx<T>::type* four;         // [NFOURIER][M+1][B][J] state read by the step
  typename cplx<T>::type* four_out;     // state written by the step (== four for in place)
  const double* par;                    // [NPAR][B]
  double* member;                       // [NMEMBER][B]
  double* diag;                         // [steps+1][NDIAG][B] or null
  typename cplx<T>::type* lam;          // adjoint Fourier fields (adjoint launches)
  const typename cplx<T>::type* lamY;   // adjoint of the K1 outputs (adjoint launches)
  double* grad;                         // [NGRAD][B] (adjoint launches)
  const typename cplx<T>::type* four_p; // tangent-linear launches: primal state before the step
  const double* dpar;                   // tangent-linear launches: [NTANGENT][B] parameter tangents
  // primal step of a tangent run with filter-weight tangents (cfg.tl_filter):
  // the tangent Fourier state and the tangents of the residual weights [2][B]
  typename cplx<T>::type* four_t;
  double* dw;
  const T* nco;                         // coefficient tables of the call (CoefTables)
  const T* jco;
  const T* djco;
  const T* mco;
};

// Work counter of a persistent launch: units are taken in turn by CTAs that
// stay resident; the last CTA out resets both words for the next launch on
// the same stream.
struct SchedCounter {
  int next;
  int done;
};

template <typename T>
struct SpecLaunch {
  SpecGroup<T> grp[MAXG];
  int ng;
  int prefix[MAXG + 1];
  StepCfg cfg;
  int mode;                             // 0 = step, 2 = diagnose winds, 3 = tangent-linear step
  // persistent scheduling (SIMT kernels): when sched is set the launch has one
  // CTA per resident slot, which take units in order of decreasing truncation
  // (sorder: groups by decreasing M; sprefix: unit offsets in that order)
  SchedCounter* sched;
  int sorder[MAXG];
  int sprefix[MAXG + 1];
};

// ------------------------------------------------------------------- grid ---
template <typename T>
struct GridGroup {
  Geom<T> g;
  int B, JB, njb;                       // members, rows per CTA, row-blocks per member
  typename cplx<T>::type* four;         // [NFOURIER][M+1][B][J]
  T* resid;                             // [NRESID][B][J][I]
  const double* par;                    // [NPAR][B]
  double* member;                       // [NMEMBER][B]
  double* diag;                         // [steps+1][NDIAG][B] or null
  T* hist;                              // [5][B][J][I] for this step, or null
  const T* phys_in;                     // init: [5][B][J][I] physical initial fields
  T* phys_out;                          // output/adjoint: [5 or 8][B][J][I]
  // adjoint
  typename cplx<T>::type* lam;          // adjoint Fourier fields
  typename cplx<T>::type* lamy;         // adjoint of the K1 outputs [5][M+1][B][J]
  const typename cplx<T>::type* primal; // primal Fourier fields after the step
  double* grad;                         // [NGRAD][B]
  // tangent-linear
  const T* phys_p;                      // primal physical ICs (tangent init)
  const double* dpar;                   // [NTANGENT][B] parameter tangents
  const T* resid_p;                     // primal IC residual (tangent step and output)
  const double* dw;                     // tangents of the residual weights [2][B] (tangent step and output)
};

template <typename T>
struct GridLaunch {
  GridGroup<T> grp[MAXG];
  int ng;
  int prefix[MAXG + 1];
  StepCfg cfg;
  int mode;
};

enum GridMode {
  GM_STEP = 0,       // Fourier (eta, Phi, U, V) -> nonlinear Fourier terms (+history, diagnostics)
  GM_INIT = 1,       // physical ICs -> full Fourier state, residuals, diagnostics
  GM_OUTPUT = 2,     // Fourier state -> physical curr/prev fields
  GM_WINDS = 3,      // Fourier U, V -> physical U, V (diagnosed winds)
  GM_ADJ_STEP = 4,   // adjoint of GM_STEP
  GM_ADJ_INIT = 5,   // adjoint of GM_INIT (gradient w.r.t. physical ICs)
  GM_ADJ_OUTPUT = 6, // adjoint of the physical curr fields of GM_OUTPUT
  GM_FWD2 = 7,       // physical eta, delta -> truncated Fourier (diagnosed winds)
  GM_TL_STEP = 8,    // tangent of GM_STEP (linearised nonlinear terms and forcing)
  GM_TL_INIT = 9,    // tangent of GM_INIT
  NGRIDMODE = 10
};

// Launch of a step kernel with programmatic stream serialization (see
// pdl_enter): on for the FP32 kernels unless the environment sets SWP_PDL=0.
// The FP64 kernels launch plainly: measured, the attribute cost the
// single-member FP64 drop-in run 15% and gained nothing at 64 members.
bool pdl_enabled();
template <typename... Params, typename... Args>
cudaError_t launch_pdl(void (*kernel)(Params...), int nblocks, int threads, size_t smem, cudaStream_t s,
                       bool fp32, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nblocks);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = (fp32 && pdl_enabled()) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <typename T> size_t spec_smem_bytes(int M, int J, int MT);
template <typename T> size_t spec_adj_smem_bytes(int M, int J, int MT);
template <typename T> size_t grid_smem_bytes(int M, int J, int I, int JB, int mode);
template <typename T> cudaError_t launch_spec(const SpecLaunch<T>& L, int nblocks, size_t smem, cudaStream_t s);
template <typename T> cudaError_t launch_spec_adj(const SpecLaunch<T>& L, int nblocks, size_t smem, cudaStream_t s);
template <typename T> cudaError_t launch_grid(const GridLaunch<T>& L, int nblocks, size_t smem, cudaStream_t s);
void spec_set_attributes();
// dynamic shared memory a SIMT Legendre kernel may use (the rest of the 227 KB
// is kept for its static shared memory)
constexpr int SPEC_DYN_SMEM_MAX = 227 * 1024 - 128;
void grid_set_attributes();
int grid_rows_per_cta(int M, bool fp64, int mode);  // JB the grid kernel is compiled for

// tensor-core Legendre kernels of the FP32 modified-Euler step and its adjoint
// (tc_legendre.cu: M = 42 and 63; tc_legendre106.cu: M = 106)
// packed basis of each group, and the poll limit of the kernels' mbarrier waits
struct TcBasis {
  const float* p[MAXG];
  uint32_t wait_limit;
};
constexpr uint32_t TC_WAIT_LIMIT_DEFAULT = SWP_WAIT_LIMIT_DEFAULT;
size_t spec_tc_smem_bytes(int M);
size_t spec_tc_basis_floats(int M);
int spec_tc_members_per_cta();
bool spec_tc_supported(int M);      // forward kernel
bool spec_tc_adj_supported(int M);  // adjoint kernel
size_t spec_tc_adj_basis_floats(int M);
int pack_tc_basis(const GroupGeom& gg, float* out, cudaStream_t s);
void spec_tc_set_attributes();
cudaError_t launch_spec_tc(int M, const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                           cudaStream_t s);
int pack_tc_basis_adj(const GroupGeom& gg, float* out, cudaStream_t s);
size_t spec_tc_adj_smem_bytes(int M);
cudaError_t launch_spec_adj_tc(int M, const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                               cudaStream_t s);
size_t spec_tc106_smem_bytes();
size_t spec_tc106_adj_smem_bytes();
size_t spec_tc106_basis_floats();
int pack_tc106_basis(const GroupGeom& gg, float* out, bool adjoint, cudaStream_t s);
void spec_tc106_set_attributes();
cudaError_t launch_spec_tc106(const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                              cudaStream_t s);
cudaError_t launch_spec_adj_tc106(const SpecLaunch<float>& L, int nblocks, const TcBasis& basis, int* err,
                                  cudaStream_t s);

}  // namespace swp
