// Context, C ABI and host-side drivers of the GB300 FFT-PEEC path.
//
// The context owns one geometry on one GPU: lattice maps, spectra, topology lists,
// per-frequency operator state (DZ, Yle, LU factors) and the Krylov workspace.
// Host code only sequences kernels and runs the small dense parts of GMRES
// (Givens rotations, triangular solves on <= maxit unknowns) in FP64.
#include <algorithm>
#include <array>
#include <map>
#include <queue>
#include <mutex>
#include <new>
#include <stdexcept>
#include <tuple>
#include <cmath>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "ctx.hpp"
#include "peec_gb300.h"

namespace peec {

// NVTX ranges around the C-ABI entry points (header-only NVTX 3: no cost unless a
// profiler attaches), so a timeline shows fill, frequency set-up and solves per context
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }

static int badarg(const char* fn) {
  g_err = std::string(fn) + ": null pointer or argument out of range";
  return PEEC_ERR_BADARG;
}
int fail_cuda(cudaError_t e, const char* expr, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "CUDA error %s (%d) at %s:%d in %s", cudaGetErrorString(e), (int)e,
           file, line, expr);
  g_err = buf;
  return e == cudaErrorMemoryAllocation ? PEEC_ERR_OOM : PEEC_ERR_CUDA;
}

// launchers defined in the other translation units
void launch_edge_rows(const c64*, const c64*, const c64*, const c64*, const int32_t*,
                      const int32_t*, const double*, int, c64*, c64*, cudaStream_t);
void launch_surf_rows(const c64*, const c64*, const int32_t*, const double*, int, c64*, c64*,
                      cudaStream_t);
void launch_node_rows(const c64*, const c64*, const c64*, const c64*, const c64*, const int32_t*,
                      const int32_t*, const int32_t*, const int32_t*, const int32_t*,
                      const int32_t*, const c64*, const double*, int, c64*, cudaStream_t);
void launch_set_scalar(double* p, double v, cudaStream_t st);
void launch_edge_dz(int64_t m, const double* R4, const double* Cd4, const double* Lpd,
                    const double* Zs0, const uint8_t* surf, double escal_R, double sq, double w,
                    c64* DZ, cudaStream_t st);
int dense_chunks(int64_t n);
int64_t dense_ld(int64_t n);
int dense_apply(const void* M, bool fp32, int64_t n, int64_t ld, const c64* x, int offdiag,
                c64* part, c64* out, cudaStream_t st);
void dense_round(const double* a, size_t cnt, float* out, cudaStream_t st);
int64_t dense_part_c(int64_t n);
int dense_apply_c(const void* M, bool fp32, int64_t n, int64_t ld, const c64* x, int offdiag,
                  c64* part, c64* out, cudaStream_t st);
void dense_phase(const double* M, const double* R, size_t cnt, double beta, c64* Mc, c32* Mc32,
                 cudaStream_t st);
void launch_final_rows(const c64*, const c64*, const c64*, const c64*, const int32_t*,
                       const int32_t*, const int32_t*, const double*, int, int, int, c64*,
                       cudaStream_t);
void launch_perm_gather(const c64*, const int32_t*, const double*, int, c64*, cudaStream_t);
int sptrsv_grp_prepare(size_t smem_bytes);
int launch_sptrsv(const GrpPlan&, cudaStream_t, cudaEvent_t, cudaEvent_t, const int32_t*, int,
                  int, const SfTri&, const SfTri&,
                  const c64*, const int32_t*, const double*, c64*, c64*, int*, cudaStream_t);
int red_blocks(size_t N);
int launch_multidot(const c64*, size_t, const c64*, size_t, int, c64*, c64*, cudaStream_t);
int launch_multidot(const cff*, size_t, const c64*, size_t, int, c64*, c64*, cudaStream_t);
int launch_multidot(const cff*, size_t, const cff*, size_t, int, c64*, c64*, cudaStream_t);
void launch_multiaxpy(const c64*, size_t, const c64*, int, const c64*, int, size_t, c64*, size_t,
                      double*, cudaStream_t);
void launch_multiaxpy(const cff*, size_t, const c64*, int, const c64*, int, size_t, c64*, size_t,
                      double*, cudaStream_t);
void launch_norm2(const c64*, size_t, size_t, double*, double*, cudaStream_t);
void launch_sum_parts(const double*, int, double*, cudaStream_t);
void launch_scale_rnorm(c64*, size_t, const double*, cudaStream_t);
void launch_make_reflector(const c64*, size_t, int, c64, double, c64*, cudaStream_t);
void launch_make_reflector(const c64*, size_t, int, c64, double, cff*, cudaStream_t);
void launch_sub(const c64*, const c64*, size_t, c64*, cudaStream_t);
void launch_add(const c64*, const c64*, size_t, c64*, cudaStream_t);
void launch_add_i(const c64*, size_t, c64*, cudaStream_t);
void launch_differs(const c64*, const c64*, size_t, int*, cudaStream_t);
void launch_tri(c64*, int, int, const c64*, c64*, int, cudaStream_t);
void launch_xupdate(const c64*, const c64*, size_t, const c64*, const c64*, int, size_t, c64*,
                    cudaStream_t);
void launch_xupdate(const c64*, const cff*, size_t, const c64*, const c64*, int, size_t, c64*,
                    cudaStream_t);
int fill_rows_rcc_gpu(const double origin[3], double sx, double sy, double sz, double escal_Lp,
                      double escal_P, int Nx, int Ny, int Nz, double* const d_rows[9],
                      const int64_t row_len[9], int* d_bad, cudaStream_t st);
int rcc_rows_gpu(const double origin[3], double sx, double sy, double sz, int Nx, int Ny, int Nz,
                 double beta, const double* const d_qs[9], double* const d_re[9],
                 double* const d_im[9], const int64_t row_len[9], cudaStream_t st);
int fill_rows_gpu(const double origin[3], double sx, double sy, double sz, double escal_Lp,
                  double escal_P, int Nx, int Ny, int Nz, double* const d_rows[9],
                  const int64_t row_len[9], int* d_bad, cudaStream_t st);
size_t ris_box_bytes();
int ris_prep_gpu(int surfaces, const double* d_geom, int64_t count, int64_t mx, int64_t my,
                 void* boxes, double* self, int* nrm, cudaStream_t st);
int ris_pairs_gpu(int kind, int nb, const void* const* boxes, const int* nrm,
                  const double* const* S, const double* const* self, const int64_t* dim,
                  double esc, double* const* M, const int64_t* ld, int* d_bad, cudaStream_t st);
int ris_dist_gpu(const double* d_ctr, int64_t dim, double* R, int64_t ld, cudaStream_t st);
int inv_diag_gpu(const double* M, int64_t ld, int64_t n, double* inv, cudaStream_t st);
void launch_adjoint(const c64*, const int32_t*, const int32_t*, const c64*, const c64*, double,
                    int64_t, int64_t, double*, cudaStream_t);
int selftest_wait_limit(int limit, cudaStream_t st, int* err_out);

}  // namespace peec

using namespace peec;
using cd = std::complex<double>;

struct LevelTri {  // triangular factor without its diagonal (CSR) and its level sets
  int32_t *ptr = nullptr, *col = nullptr, *flag = nullptr;
  c64 *val = nullptr, *dinv = nullptr;
  int64_t nflag = 0;
  std::vector<int32_t> rows;     // rows sorted by level (host)
  std::vector<int> lvl_off;      // offsets into rows per level (host)
  std::vector<int32_t> hptr, hcol;  // host copy of the structure
};

struct peec_ctx {
  int dev = 0;
  cudaStream_t st = nullptr;
  // a second stream for the LU solve's large groups (forked from st and joined back with
  // the two events, so the packed groups run beside them)
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::string err;
  int64_t launches = 0;
  // twiddle master tables
  int twmax = 0;
  void* tw64 = nullptr;
  void* tw32 = nullptr;
  void* twff = nullptr;
  int resid_prec = PEEC_PREC_FF;  // arithmetic of the refinement residuals
  // sizes
  int Nx = 0, Ny = 0, Nz = 0;
  int64_t mx = 0, my = 0, mz = 0, m = 0, ns = 0, n = 0, N = 0;
  bool have_topo = false, have_spec = false, have_freq = false, have_pdiag = false;
  // lattice: the topology has voxel lattices (circulant operator); dense: the operator's
  // Lp and P products come from dense matrices (the RIS solver): Lp_x, Lp_y, Lp_z, P,
  // real column-major, FP64 and an FP32 copy, and the scratch of their partial sums
  bool lattice = false, dense = false;
  double* dn64[4] = {nullptr, nullptr, nullptr, nullptr};
  int64_t dn_ld[4] = {4, 4, 4, 4};  // padded leading dimensions
  float* dn32[4] = {nullptr, nullptr, nullptr, nullptr};
  // partial sums of the chunked products: the Lp blocks (one after another on st2) use the
  // first dn_part_half entries, P (on st, beside them) the second
  c64* dn_part = nullptr;
  size_t dn_part_half = 0;
  // the dense retarded operator (peec_set_dense_rcc): centre distances R per block, and the
  // blocks times exp(-j beta R) of the installed frequency (FP64 and FP32 copies)
  bool dense_rcc = false, dense_rcc_ready = false;
  double* dnR[4] = {nullptr, nullptr, nullptr, nullptr};
  // which blocks hold a matrix / distances (peec_set_dense, peec_set_dense_rcc, peec_ris_fill)
  bool dn_set[4] = {false, false, false, false};
  bool dnR_set[4] = {false, false, false, false};
  c64* dnc64[4] = {nullptr, nullptr, nullptr, nullptr};
  c32* dnc32[4] = {nullptr, nullptr, nullptr, nullptr};
  // topology
  int32_t *n1 = nullptr, *n2 = nullptr, *snode = nullptr;
  double* invP = nullptr;
  int32_t *ne_ptr = nullptr, *ne_idx = nullptr, *nsn_ptr = nullptr, *nsn_idx = nullptr;
  Family fam[6];
  Spectrum spec[9];
  void* ph64[3] = {nullptr, nullptr, nullptr};  // face-grid phase tables (octant spectra)
  void* ph32[3] = {nullptr, nullptr, nullptr};  // their FP32 rounding (FP32 z passes)
  int* zerr = nullptr;  // set by a staged z pass whose copy wait ran into its limit
  int nsm = 0;          // SM count of the device
  ZTune zt;             // FP32 z-pass forms chosen by the tuner for this context's grids
  double zface_ms[3] = {-1, -1, -1};          // tuner times per face form (-1: not a candidate)
  double zedge_ms[6] = {-1, -1, -1, -1, -1, -1};  // per edge plan x form
  int row_dims[9][3] = {};
  // retarded (Rcc, solverType 2) operator: the QS parts of its nine rows (escaled), the
  // lattice geometry of the centre distances, and at the current frequency the spectra of
  // the rows' imaginary parts (spec then holds those of the real parts); operator
  // applications run both convolutions and join them (rcc set)
  double* rcc_qs[9] = {};
  double rcc_origin[3] = {0, 0, 0}, rcc_s[3] = {0, 0, 0};
  bool have_rcc_rows = false, rcc = false;
  double rcc_freq = -1.0;
  Spectrum spec_im[9];
  c64 *LpI2 = nullptr, *PQ2 = nullptr;
  // frequency state
  double w = 0.0;
  c64* DZ = nullptr;
  int32_t *yle_ptr = nullptr, *yle_col = nullptr;
  c64* yle_val = nullptr;
  int32_t *g_in = nullptr, *g_out = nullptr;  // LU permutations as gathers
  double* lu_rs = nullptr;                    // optional row scaling of the LU
  // synchronisation-free triangular solves: claim order (L levels then U levels, each
  // padded with -1 to whole warps), its length, the L part's length, control words
  int32_t* sf_ord = nullptr;
  // per-warp group solves (GrpPlan): components of at most comp_max rows; the device
  // arrays of the plan (host-built with the factors' structure)
  int comp_max = SF_COMP_MAX;  // largest component solved per warp (0: global scheme only)
  GrpPlan grp;
  int32_t *grp_goff = nullptr, *grp_seg = nullptr, *grp_segoff = nullptr, *grp_nsegL = nullptr;
  GrpRow* grp_rows = nullptr;
  int16_t *grp_uq = nullptr, *grp_lcolL = nullptr, *grp_lcolU = nullptr;
  c64 *ir_b = nullptr, *ir_x = nullptr, *ir_r = nullptr, *ir_d = nullptr;  // refinement vectors
  // the frequency w on the device (the row kernels read it there, so captured graphs of
  // the operator stay valid when only the frequency state changes) and the entries the
  // Yle value array holds
  double* d_w = nullptr;
  size_t yle_cap = 0;
  // per-edge data of the device frequency state (peec_set_edge_state): R and Cd of the four
  // edge halves, Lp self terms, the surface-impedance base and the surface-edge flags
  double *es_R4 = nullptr, *es_Cd4 = nullptr, *es_Lpd = nullptr, *es_Zs0 = nullptr;
  uint8_t* es_surf = nullptr;
  double es_escal_R = 1.0, es_escal_freq = 1.0;
  bool have_es = false;
  // convolutions of the last converged mixed solve's final residual: x, Lp*I, P*Q and
  // the precision they were computed in (-1: none). They do not depend on the frequency.
  c64 *cc_x = nullptr, *cc_LpI = nullptr, *cc_PQ = nullptr;
  int cc_prec = -1;
  int* d_flag = nullptr;
  int sf_total = 0, sf_nL = 0;
  int* sf_ctl = nullptr;  // [epoch, claim counter, error flag]
  LevelTri Lf, Uf;
  // device refactorisation of SS in the current factors' pattern (refactor.cu)
  RefactorPlan rf;
  bool have_rf = false;
  std::vector<int32_t> h_gin, h_gout;   // host copies of the LU row / column gathers
  std::vector<int32_t> rf_yp, rf_yc;    // the Yle pattern (CSR) the plan was built for
  int* rf_err = nullptr;
  // matvec work
  c64 *LpI = nullptr, *PQ = nullptr, *Y1 = nullptr, *U1 = nullptr, *Y2 = nullptr, *U2 = nullptr;
  c64 *tvec = nullptr, *Mvec = nullptr, *lutmp = nullptr, *lutmp2 = nullptr;
  // host staging
  c64 *hx = nullptr, *hy = nullptr;  // pinned N
  c64 *dx = nullptr, *dy = nullptr;  // device N
  // krylov workspace
  int kcap = 0;
  c64* U = nullptr;     // reflector basis of the FP64 / float-float solves, N x kcap_u
  cff* U32 = nullptr;   // reflector basis of the FP32-operator (inner) solves, float-float, N x kcap_u32
  int kcap_u = 0, kcap_u32 = 0;
  c64 *gb = nullptr, *gx = nullptr, *gr = nullptr, *gv = nullptr, *gw = nullptr, *gxm = nullptr,
      *gxmin = nullptr, *gtmp = nullptr, *gzero = nullptr;
  c64 *dcoef = nullptr, *dcoef2 = nullptr, *dpart = nullptr, *dT = nullptr;
  double *dred = nullptr, *dscal = nullptr;
  c64* hsmall = nullptr;  // pinned staging ring for host -> device coefficients
  c64* hread = nullptr;   // pinned staging for device -> host reads
  double* hscal = nullptr;
  volatile int* stop = nullptr;
  float t_total = 0, t_conv = 0, t_sparse = 0;
  // per-class profiling (peec_profile_matvec)
  bool prof = false;
  std::vector<cudaEvent_t> pev;
  double prof_ms[5] = {0, 0, 0, 0, 0};
  // scratch of peec_multidot
  c64* mdpart = nullptr;
  size_t mdcap = 0;
  // CUDA graphs of operator applications, keyed by (x, y, precision); captured on the
  // second application with the same key, dropped whenever operator state changes
  struct GraphEntry {
    int calls = 0;
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
  };
  std::map<std::tuple<const void*, void*, int>, GraphEntry> graphs;
  bool use_graphs = true;
  // device-resident Arnoldi loop: the cycle state (GmDev header, res, wv, J, Utop, R) in
  // one allocation for cycles of gm_inner iterations, its pinned mirrors (gm_up: the
  // header, gm_down: header + res + wv), and per operator precision a graph whose WHILE
  // node runs iterations until the scalar step ends the loop
  unsigned char* gm_block = nullptr;
  unsigned char* gm_up = nullptr;
  unsigned char* gm_down = nullptr;
  int gm_inner = -1;
  struct KrylovGraph {
    cudaGraphExec_t exec = nullptr;
    int inner = -1;
    int64_t kernels = 0;  // kernels per iteration
  };
  KrylovGraph kg[3];
  bool dev_loop = true;
  int64_t kg_launches = 0, kg_iterations = 0;
};

static void drop_krylov_graphs(peec_ctx* ctx) {
  for (auto& k : ctx->kg) {
    if (k.exec) cudaGraphExecDestroy(k.exec);
    k = peec_ctx::KrylovGraph();
  }
}

static void drop_graphs(peec_ctx* ctx) {
  if (!ctx) return;
  for (auto& kv : ctx->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  ctx->graphs.clear();
  drop_krylov_graphs(ctx);
}

// Entry points make the context's device current for their work; this puts the
// caller's current device back on return, so a caller mixing contexts of several
// devices with its own device-current work is not switched underneath.
struct DeviceRestore {
  int dev = -1;
  DeviceRestore() noexcept {
    if (cudaGetDevice(&dev) != cudaSuccess) {
      dev = -1;
      cudaGetLastError();
    }
  }
  ~DeviceRestore() {
    if (dev >= 0) cudaSetDevice(dev);
  }
};

#define CTX_TRY(expr)                 \
  do {                                \
    int _rc = (expr);                 \
    if (_rc != PEEC_OK) {             \
      ctx->err = g_err;               \
      return _rc;                     \
    }                                 \
  } while (0)
#define CTX_CUDA(expr) CTX_TRY(([&]() -> int { PEEC_CUDA_TRY(expr); return PEEC_OK; })())

static int bad(peec_ctx* ctx, int code, const std::string& msg) {
  ctx->err = msg;
  g_err = msg;
  return code;
}

template <typename T>
static int dalloc(T** p, size_t count) {
  if (*p) {
    cudaFree(*p);
    *p = nullptr;
  }
  if (count == 0) count = 1;
  PEEC_CUDA_TRY(cudaMalloc((void**)p, count * sizeof(T)));
  return PEEC_OK;
}

template <typename T>
static int upload(T** p, const std::vector<T>& h, cudaStream_t st) {
  int rc = dalloc(p, h.size());
  if (rc) return rc;
  if (!h.empty()) PEEC_CUDA_TRY(cudaMemcpyAsync(*p, h.data(), h.size() * sizeof(T),
                                                cudaMemcpyHostToDevice, st));
  return PEEC_OK;
}

static int pow2ceil(int v) {
  int r = 1;
  while (r < v) r <<= 1;
  return r;
}

extern "C" int peec_version(void) { return 100; }

// The calling thread's most recent error wins: every failing entry point records its
// message there, including CUDA failures deep inside a launch sequence.
extern "C" const char* peec_last_error(const peec_ctx* ctx) {
  if (!ctx || !g_err.empty()) return g_err.c_str();
  return ctx->err.c_str();
}

extern "C" int64_t peec_launch_count(const peec_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" int peec_sizes(const peec_ctx* ctx, int64_t* m, int64_t* ns, int64_t* n) {
  if (!ctx) return badarg(__func__);
  if (m) *m = ctx->m;
  if (ns) *ns = ctx->ns;
  if (n) *n = ctx->n;
  return PEEC_OK;
}

static int peec_ctx_create_body(peec_ctx** out, int device) {
  if (!out) return badarg("peec_ctx_create");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    g_err = std::string("no CUDA device available: ") + cudaGetErrorString(e);
    return PEEC_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) {
    g_err = "device index out of range";
    return PEEC_ERR_BADARG;
  }
  peec_ctx* ctx = new peec_ctx();
  ctx->dev = device;
  auto fail = [&](int rc) {
    peec_ctx_destroy(ctx);
    return rc;
  };
  if (cudaSetDevice(device) != cudaSuccess) return fail(fail_cuda(cudaGetLastError(), "cudaSetDevice", __FILE__, __LINE__));
  if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->st2, cudaStreamNonBlocking) != cudaSuccess)
    return fail(fail_cuda(cudaGetLastError(), "cudaStreamCreate", __FILE__, __LINE__));
  if (cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess)
    return fail(fail_cuda(cudaGetLastError(), "cudaEventCreate", __FILE__, __LINE__));
  for (auto& ev : ctx->ev) cudaEventCreate(&ev);
  // twiddle master table exp(-2 pi i e / twmax), long-double accurate
  ctx->twmax = 8192;
  std::vector<c64> t64(ctx->twmax);
  std::vector<c32> t32(ctx->twmax);
  std::vector<cff> tff(ctx->twmax);
  // float-float split of a long double: hi the nearest float, lo the nearest float of
  // the remainder
  auto split = [](long double v) {
    const float h = (float)v;
    return ff(h, (float)(v - (long double)h));
  };
  for (int e = 0; e < ctx->twmax; ++e) {
    long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)e /
                    (long double)ctx->twmax;
    t64[e] = mk<double>((double)cosl(a), (double)sinl(a));
    t32[e] = mk<float>((float)cosl(a), (float)sinl(a));
    tff[e] = mk<ff>(split(cosl(a)), split(sinl(a)));
  }
  if (cudaMalloc(&ctx->tw64, sizeof(c64) * ctx->twmax) != cudaSuccess ||
      cudaMalloc(&ctx->tw32, sizeof(c32) * ctx->twmax) != cudaSuccess ||
      cudaMalloc(&ctx->twff, sizeof(cff) * ctx->twmax) != cudaSuccess)
    return fail(fail_cuda(cudaErrorMemoryAllocation, "cudaMalloc twiddles", __FILE__, __LINE__));
  cudaMemcpy(ctx->tw64, t64.data(), sizeof(c64) * ctx->twmax, cudaMemcpyHostToDevice);
  cudaMemcpy(ctx->tw32, t32.data(), sizeof(c32) * ctx->twmax, cudaMemcpyHostToDevice);
  cudaMemcpy(ctx->twff, tff.data(), sizeof(cff) * ctx->twmax, cudaMemcpyHostToDevice);
  if (cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return fail(fail_cuda(cudaGetLastError(), "cudaDeviceGetAttribute", __FILE__, __LINE__));
  if (cudaMalloc(&ctx->zerr, sizeof(int)) != cudaSuccess ||
      cudaMemset(ctx->zerr, 0, sizeof(int)) != cudaSuccess)
    return fail(fail_cuda(cudaErrorMemoryAllocation, "cudaMalloc error word", __FILE__, __LINE__));
  cudaMallocHost(&ctx->hsmall, sizeof(c64) * 16 * 4096);
  cudaMallocHost(&ctx->hread, sizeof(c64) * 4096);
  cudaMallocHost(&ctx->hscal, sizeof(double) * 64);
  *out = ctx;
  return PEEC_OK;
}

static void free_refactor(RefactorPlan& r) {
  cudaFree(r.asm_ptr); cudaFree(r.asm_src); cudaFree(r.rows); cudaFree(r.upd_off);
  cudaFree(r.upd_tgt); cudaFree(r.D);
  r = RefactorPlan();
}

static void free_tri(LevelTri& t) {
  cudaFree(t.ptr); cudaFree(t.col); cudaFree(t.val); cudaFree(t.dinv); cudaFree(t.flag);
  t = LevelTri();
}

extern "C" void peec_ctx_destroy(peec_ctx* ctx) {
  if (!ctx) return;
  DeviceRestore restore_device_;
  cudaSetDevice(ctx->dev);
  if (ctx->st) cudaStreamSynchronize(ctx->st);
  drop_graphs(ctx);
  void* ptrs[] = {ctx->tw64, ctx->tw32, ctx->twff, ctx->n1, ctx->n2, ctx->snode, ctx->invP, ctx->ne_ptr,
                  ctx->ne_idx, ctx->nsn_ptr, ctx->nsn_idx, ctx->DZ, ctx->yle_ptr, ctx->yle_col,
                  ctx->yle_val, ctx->g_in, ctx->g_out, ctx->lu_rs, ctx->LpI, ctx->PQ, ctx->Y1, ctx->U1,
                  ctx->Y2, ctx->U2, ctx->tvec, ctx->Mvec, ctx->lutmp, ctx->lutmp2, ctx->dx, ctx->dy, ctx->U, (c64*)ctx->U32,
                  ctx->gb, ctx->gx, ctx->gr, ctx->gv, ctx->gw, ctx->gxm, ctx->gxmin, ctx->gtmp,
                  ctx->gzero, ctx->dcoef, ctx->dcoef2, ctx->dpart, ctx->dred, ctx->dscal, ctx->dT,
                  ctx->mdpart, ctx->LpI2, ctx->PQ2, ctx->gm_block, ctx->d_w, ctx->dn_part,
                  ctx->dn64[0], ctx->dn64[1], ctx->dn64[2], ctx->dn64[3], ctx->dn32[0],
                  ctx->dn32[1], ctx->dn32[2], ctx->dn32[3], ctx->dnR[0], ctx->dnR[1],
                  ctx->dnR[2], ctx->dnR[3], ctx->dnc64[0], ctx->dnc64[1], ctx->dnc64[2],
                  ctx->dnc64[3], ctx->dnc32[0], ctx->dnc32[1], ctx->dnc32[2], ctx->dnc32[3],
                  ctx->es_R4, ctx->es_Cd4,
                  ctx->es_Lpd, ctx->es_Zs0, ctx->es_surf};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (ctx->gm_up) cudaFreeHost(ctx->gm_up);
  if (ctx->gm_down) cudaFreeHost(ctx->gm_down);
  for (double* p : ctx->rcc_qs)
    if (p) cudaFree(p);
  for (auto& f : ctx->fam) {
    if (f.map) cudaFree(f.map);
    for (int p = 0; p < 2; ++p)
      if (f.T[p]) cudaFree(f.T[p]);
  }
  for (Spectrum* set : {ctx->spec, ctx->spec_im})
    for (int i = 0; i < 9; ++i) {
      Spectrum& s = set[i];
      for (int p = 0; p < 2; ++p)
        if (s.d[p]) cudaFree(s.d[p]);
      if (s.oct) cudaFree(s.oct);
      if (s.yz32) cudaFree(s.yz32);
    }
  for (int a = 0; a < 3; ++a) {
    if (ctx->ph64[a]) cudaFree(ctx->ph64[a]);
    if (ctx->ph32[a]) cudaFree(ctx->ph32[a]);
  }
  cudaFree(ctx->zerr);
  free_tri(ctx->Lf);
  free_tri(ctx->Uf);
  cudaFree(ctx->sf_ord);
  cudaFree(ctx->sf_ctl);
  free_refactor(ctx->rf);
  cudaFree(ctx->rf_err);
  for (void* p : {(void*)ctx->grp_goff, (void*)ctx->grp_seg, (void*)ctx->grp_segoff,
                  (void*)ctx->grp_nsegL, (void*)ctx->grp_rows, (void*)ctx->grp_uq,
                  (void*)ctx->grp_lcolL, (void*)ctx->grp_lcolU})
    cudaFree(p);
  for (c64* p : {ctx->ir_b, ctx->ir_x, ctx->ir_r, ctx->ir_d, ctx->cc_x, ctx->cc_LpI, ctx->cc_PQ})
    cudaFree(p);
  cudaFree(ctx->d_flag);
  if (ctx->hx) cudaFreeHost(ctx->hx);
  if (ctx->hy) cudaFreeHost(ctx->hy);
  if (ctx->hsmall) cudaFreeHost(ctx->hsmall);
  if (ctx->hread) cudaFreeHost(ctx->hread);
  if (ctx->hscal) cudaFreeHost(ctx->hscal);
  for (auto& ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto e : ctx->pev) cudaEventDestroy(e);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->st2) {
    cudaStreamSynchronize(ctx->st2);
    cudaStreamDestroy(ctx->st2);
  }
  if (ctx->st) cudaStreamDestroy(ctx->st);
  delete ctx;
}

extern "C" int peec_set_stop_flag(peec_ctx* ctx, volatile int* flag) {
  if (!ctx) return badarg(__func__);
  ctx->stop = flag;
  return PEEC_OK;
}

extern "C" int peec_set_device_loop(peec_ctx* ctx, int on) {
  if (!ctx || (on != 0 && on != 1)) return badarg(__func__);
  ctx->dev_loop = on != 0;
  return PEEC_OK;
}

extern "C" int peec_device_loop_stats(const peec_ctx* ctx, int64_t* graph_launches,
                                      int64_t* iterations) {
  if (!ctx || !graph_launches || !iterations) return badarg(__func__);
  *graph_launches = ctx->kg_launches;
  *iterations = ctx->kg_iterations;
  return PEEC_OK;
}

// ------------------------------------------------------------------------------------
// topology
// ------------------------------------------------------------------------------------

// FFT length along one dimension: a symmetric block needs L >= 2N-2, a general
// Toeplitz block L >= na+nb-1; rounded up to a power of two.
static int fft_len(int na, int nb, bool sym) {
  int need = sym ? (na > 1 ? 2 * na - 2 : 1) : na + nb - 1;
  return pow2ceil(need < 1 ? 1 : need);
}

// the sparse topology: edge end nodes (A), surface nodes (Gamma) and the node -> edge /
// node -> surface lists the row kernels gather with
static int set_incidence_lists(peec_ctx* ctx, int64_t m, int64_t ns, int64_t n,
                               const int64_t* edge_n1, const int64_t* edge_n2,
                               const int64_t* surf_node) {
  std::vector<int32_t> hn1(m), hn2(m), hsn(ns);
  std::vector<int32_t> deg(n + 1, 0), sdeg(n + 1, 0);
  for (int64_t e = 0; e < m; ++e) {
    if (edge_n1[e] < 0 || edge_n1[e] >= n || edge_n2[e] < 0 || edge_n2[e] >= n)
      return bad(ctx, PEEC_ERR_BADARG, "edge node out of range");
    hn1[e] = (int32_t)edge_n1[e];
    hn2[e] = (int32_t)edge_n2[e];
    deg[hn1[e] + 1]++;
    deg[hn2[e] + 1]++;
  }
  for (int64_t s = 0; s < ns; ++s) {
    if (surf_node[s] < 0 || surf_node[s] >= n) return bad(ctx, PEEC_ERR_BADARG, "surface node out of range");
    hsn[s] = (int32_t)surf_node[s];
    sdeg[hsn[s] + 1]++;
  }
  for (int64_t v = 0; v < n; ++v) {
    deg[v + 1] += deg[v];
    sdeg[v + 1] += sdeg[v];
  }
  std::vector<int32_t> nei(deg[n]), nsi(sdeg[n]);
  {
    std::vector<int32_t> fill(deg.begin(), deg.end() - 1);
    for (int64_t e = 0; e < m; ++e) {
      nei[fill[hn1[e]]++] = (int32_t)(2 * e);      // A = -1
      nei[fill[hn2[e]]++] = (int32_t)(2 * e + 1);  // A = +1
    }
    std::vector<int32_t> sf(sdeg.begin(), sdeg.end() - 1);
    for (int64_t s = 0; s < ns; ++s) nsi[sf[hsn[s]]++] = (int32_t)s;
  }
  CTX_TRY(upload(&ctx->n1, hn1, ctx->st));
  CTX_TRY(upload(&ctx->n2, hn2, ctx->st));
  CTX_TRY(upload(&ctx->snode, hsn, ctx->st));
  CTX_TRY(upload(&ctx->ne_ptr, deg, ctx->st));
  CTX_TRY(upload(&ctx->ne_idx, nei, ctx->st));
  CTX_TRY(upload(&ctx->nsn_ptr, sdeg, ctx->st));
  CTX_TRY(upload(&ctx->nsn_idx, nsi, ctx->st));
  return PEEC_OK;
}

// work vectors and staging of an operator with the context's sizes
static int alloc_work(peec_ctx* ctx) {
  const int64_t m = ctx->m, ns = ctx->ns, n = ctx->n;
  CTX_TRY(dalloc(&ctx->LpI, m));
  CTX_TRY(dalloc(&ctx->PQ, ns));
  CTX_TRY(dalloc(&ctx->LpI2, m));
  CTX_TRY(dalloc(&ctx->PQ2, ns));
  CTX_TRY(dalloc(&ctx->Y1, m));
  CTX_TRY(dalloc(&ctx->U1, m));
  CTX_TRY(dalloc(&ctx->Y2, ns));
  CTX_TRY(dalloc(&ctx->U2, ns));
  CTX_TRY(dalloc(&ctx->tvec, n));
  CTX_TRY(dalloc(&ctx->Mvec, n));
  CTX_TRY(dalloc(&ctx->lutmp, n));
  CTX_TRY(dalloc(&ctx->lutmp2, n));
  CTX_TRY(dalloc(&ctx->dx, ctx->N));
  CTX_TRY(dalloc(&ctx->dy, ctx->N));
  for (c64** p : {&ctx->ir_b, &ctx->ir_x, &ctx->ir_r, &ctx->ir_d, &ctx->cc_x}) CTX_TRY(dalloc(p, ctx->N));
  CTX_TRY(dalloc(&ctx->cc_LpI, m));
  CTX_TRY(dalloc(&ctx->cc_PQ, ns));
  CTX_TRY(dalloc(&ctx->d_flag, 1));
  ctx->cc_prec = -1;
  if (ctx->hx) cudaFreeHost(ctx->hx);
  if (ctx->hy) cudaFreeHost(ctx->hy);
  PEEC_CUDA_TRY(cudaMallocHost(&ctx->hx, sizeof(c64) * ctx->N));
  PEEC_CUDA_TRY(cudaMallocHost(&ctx->hy, sizeof(c64) * ctx->N));
  ctx->kcap = 0;
  ctx->have_topo = true;
  ctx->have_spec = ctx->have_freq = ctx->have_pdiag = false;
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return PEEC_OK;
}

static int peec_set_topology_body(peec_ctx* ctx, int Nx, int Ny, int Nz, int64_t mx, int64_t my,
                                 int64_t mz, const int64_t* edge_cell, const int64_t* edge_n1,
                                 const int64_t* edge_n2, int64_t ns, const int32_t* surf_fam,
                                 const int64_t* surf_cell, const int64_t* surf_node, int64_t n) {
  NvtxRange nvtx_range_("peec_set_topology");
  drop_graphs(ctx);
  if (!ctx) return badarg("peec_set_topology");
  if (Nx < 1 || Ny < 1 || Nz < 1 || mx < 0 || my < 0 || mz < 0 || ns < 0 || n < 1)
    return bad(ctx, PEEC_ERR_BADARG, "peec_set_topology: invalid sizes");
  const int64_t m = mx + my + mz;
  // device index lists are int32: unknowns, and the signed edge references 2e, 2e+1 of
  // the node-edge lists. The axis bound keeps the int lattice arithmetic (2N + 1) exact;
  // the circulant lengths are limited further by the twiddle table (below).
  if (m + ns + n > INT32_MAX || 2 * m + 1 > INT32_MAX)
    return bad(ctx, PEEC_ERR_UNSUPPORTED, "problem too large for int32 indexing");
  if (Nx > (1 << 20) || Ny > (1 << 20) || Nz > (1 << 20))
    return bad(ctx, PEEC_ERR_UNSUPPORTED, "grid axis longer than 2^20 cells");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  ctx->Nx = Nx; ctx->Ny = Ny; ctx->Nz = Nz;
  ctx->mx = mx; ctx->my = my; ctx->mz = mz; ctx->m = m; ctx->ns = ns; ctx->n = n;
  ctx->N = m + ns + n;
  // family lattices: P faces 0..2, Lp edge directions 3..5
  const int fd[6][3] = {{Nx, Ny + 1, Nz}, {Nx + 1, Ny, Nz}, {Nx, Ny, Nz + 1},
                        {Nx - 1, Ny, Nz}, {Nx, Ny - 1, Nz}, {Nx, Ny, Nz - 1}};
  std::vector<std::vector<int32_t>> maps(6);
  for (int f = 0; f < 6; ++f) maps[f].assign((size_t)fd[f][0] * fd[f][1] * fd[f][2], -1);
  const int64_t offs[4] = {0, mx, mx + my, m};
  for (int c = 0; c < 3; ++c)
    for (int64_t e = offs[c]; e < offs[c + 1]; ++e) {
      const int64_t cell = edge_cell[e];
      if (cell < 0 || cell >= (int64_t)maps[3 + c].size() || maps[3 + c][cell] != -1)
        return bad(ctx, PEEC_ERR_BADARG, "edge lattice cell out of range or duplicated");
      maps[3 + c][cell] = (int32_t)e;
    }
  for (int64_t s = 0; s < ns; ++s) {
    const int f = surf_fam[s];
    if (f < 0 || f > 2) return bad(ctx, PEEC_ERR_BADARG, "surface family out of range");
    const int64_t cell = surf_cell[s];
    if (cell < 0 || cell >= (int64_t)maps[f].size() || maps[f][cell] != -1)
      return bad(ctx, PEEC_ERR_BADARG, "surface lattice cell out of range or duplicated");
    maps[f][cell] = (int32_t)s;
  }
  for (int f = 0; f < 6; ++f) CTX_TRY(upload(&ctx->fam[f].map, maps[f], ctx->st));
  CTX_TRY(set_incidence_lists(ctx, m, ns, n, edge_n1, edge_n2, surf_node));
  // lattice families and their circulant grids: the three face families share one
  // grid (every P block, diagonal or cross, lives on it); each edge family has its own
  const int rd[9][3] = {{Nx - 1, Ny, Nz}, {Nx, Ny - 1, Nz}, {Nx, Ny, Nz - 1},
                        {Nx, Ny + 1, Nz}, {Nx + 1, Ny, Nz}, {Nx, Ny, Nz + 1},
                        {2 * Nx + 1, 2 * Ny + 1, Nz}, {Nx, 2 * Ny + 1, 2 * Nz + 1},
                        {2 * Nx + 1, Ny, 2 * Nz + 1}};
  std::memcpy(ctx->row_dims, rd, sizeof(rd));
  int LP[3];
  for (int k = 0; k < 3; ++k) {
    int need = 1;
    for (int f = 0; f < 3; ++f) need = std::max(need, fd[f][k] > 1 ? 2 * fd[f][k] - 2 : 1);
    for (int f = 0; f < 3; ++f)
      for (int g = f + 1; g < 3; ++g) need = std::max(need, fd[f][k] + fd[g][k] - 1);
    LP[k] = pow2ceil(need);
  }
  for (int f = 0; f < 6; ++f) {
    Family& F = ctx->fam[f];
    for (int p = 0; p < 2; ++p) {
      if (F.T[p]) cudaFree(F.T[p]);
      F.T[p] = nullptr;
    }
    F.lp = f >= 3;
    F.active = fd[f][0] > 0 && fd[f][1] > 0 && fd[f][2] > 0;
    for (int k = 0; k < 3; ++k) {
      F.dims[k] = fd[f][k];
      F.L[k] = f < 3 ? LP[k] : fft_len(fd[f][k], fd[f][k], true);
      F.logL[k] = ilog2(F.L[k]);
      if (F.L[k] > ctx->twmax) return bad(ctx, PEEC_ERR_UNSUPPORTED, "FFT length beyond twiddle table");
    }
    if (!F.active) continue;
    const size_t cells = (size_t)F.L[0] * F.L[1] * F.dims[2];
    PEEC_CUDA_TRY(cudaMalloc(&F.T[0], cells * sizeof(c64)));
    PEEC_CUDA_TRY(cudaMalloc(&F.T[1], cells * sizeof(c32)));
  }
  if (ctx->fam[0].L[2] * 3 * 16 * sizeof(c64) > 200 * 1024)
    return bad(ctx, PEEC_ERR_UNSUPPORTED, "z circulant too long for the z pass tile");
  for (Spectrum* set : {ctx->spec, ctx->spec_im})
    for (int i = 0; i < 9; ++i) {
      Spectrum& sp = set[i];
      for (int p = 0; p < 2; ++p) {
        if (sp.d[p]) cudaFree(sp.d[p]);
        sp.d[p] = nullptr;
      }
      if (sp.oct) cudaFree(sp.oct);
      sp.oct = nullptr;
      if (sp.yz32) cudaFree(sp.yz32);
      sp.yz32 = nullptr;
      std::memcpy(sp.L, i < 6 ? LP : ctx->fam[i - 3].L, sizeof(LP));
    }
  for (double*& p : ctx->rcc_qs) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  ctx->have_rcc_rows = ctx->rcc = false;
  ctx->rcc_freq = -1.0;
  CTX_TRY(phase_tables(LP, ctx->ph64, ctx->ph32, ctx->st));
  ctx->lattice = true;
  ctx->dense = false;
  return alloc_work(ctx);
}

// A topology without voxel lattices (the RIS solver's meshes): the incidence of the edges
// and surfaces only. The operator then needs dense Lp and P (peec_set_dense).
static int peec_set_incidence_body(peec_ctx* ctx, int64_t mx, int64_t my, int64_t mz,
                                   const int64_t* edge_n1, const int64_t* edge_n2, int64_t ns,
                                   const int64_t* surf_node, int64_t n) {
  NvtxRange nvtx_range_("peec_set_incidence");
  if (!ctx) return badarg("peec_set_incidence");
  drop_graphs(ctx);
  if (mx < 0 || my < 0 || mz < 0 || ns < 0 || n < 1 || (mx + my + mz > 0 && (!edge_n1 || !edge_n2)) ||
      (ns > 0 && !surf_node))
    return bad(ctx, PEEC_ERR_BADARG, "peec_set_incidence: invalid sizes or pointers");
  const int64_t m = mx + my + mz;
  if (m + ns + n > INT32_MAX || 2 * m + 1 > INT32_MAX)
    return bad(ctx, PEEC_ERR_UNSUPPORTED, "problem too large for int32 indexing");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  ctx->Nx = ctx->Ny = ctx->Nz = 0;
  ctx->mx = mx; ctx->my = my; ctx->mz = mz; ctx->m = m; ctx->ns = ns; ctx->n = n;
  ctx->N = m + ns + n;
  CTX_TRY(set_incidence_lists(ctx, m, ns, n, edge_n1, edge_n2, surf_node));
  for (auto& F : ctx->fam) {
    for (int p = 0; p < 2; ++p) {
      if (F.T[p]) cudaFree(F.T[p]);
      F.T[p] = nullptr;
    }
    F.active = false;
  }
  ctx->have_rcc_rows = ctx->rcc = false;
  ctx->rcc_freq = -1.0;
  ctx->lattice = false;
  ctx->dense = false;
  for (int b = 0; b < 4; ++b) ctx->dn_set[b] = ctx->dnR_set[b] = false;
  return alloc_work(ctx);
}

// Dense Lp blocks (mx x mx, my x my, mz x mz) and dense P (ns x ns), real, column-major:
// the operator's products Lp*I and P*Q become matrix-vector products with them. The
// frequency state then takes DZ = Z_self + jw diag(Lp) (the RIS solver's invZ): the
// products leave Lp's diagonal out, so that Y1 = jw Lp I + Z_self I + A Phi
// (compute_matrix_vector.jl:14-22).
static int peec_set_dense_body(peec_ctx* ctx, const double* Lpx, const double* Lpy,
                               const double* Lpz, const double* P) {
  NvtxRange nvtx_range_("peec_set_dense");
  if (!ctx) return badarg("peec_set_dense");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  const int64_t sz[4] = {ctx->mx, ctx->my, ctx->mz, ctx->ns};
  const double* src[4] = {Lpx, Lpy, Lpz, P};
  for (int b = 0; b < 4; ++b)
    if (sz[b] > 0 && !src[b]) return bad(ctx, PEEC_ERR_BADARG, "peec_set_dense: missing block");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  drop_graphs(ctx);
  ctx->dense = false;
  ctx->dense_rcc = ctx->dense_rcc_ready = false;
  size_t part = 1;
  for (int b = 0; b < 4; ++b) {
    // column-major with the leading dimension padded to a multiple of 4 (zero rows), so
    // every column starts on a 16-byte boundary for the kernels' vector loads
    const int64_t ld = dense_ld(sz[b]);
    ctx->dn_ld[b] = ld;
    const size_t cnt = (size_t)ld * (size_t)sz[b];
    CTX_TRY(dalloc(&ctx->dn64[b], cnt));
    CTX_TRY(dalloc(&ctx->dn32[b], cnt));
    if (cnt) {
      PEEC_CUDA_TRY(cudaMemsetAsync(ctx->dn64[b], 0, sizeof(double) * cnt, ctx->st));
      PEEC_CUDA_TRY(cudaMemcpy2DAsync(ctx->dn64[b], sizeof(double) * ld, src[b],
                                      sizeof(double) * sz[b], sizeof(double) * sz[b], sz[b],
                                      cudaMemcpyHostToDevice, ctx->st));
      dense_round(ctx->dn64[b], cnt, ctx->dn32[b], ctx->st);
    }
    part = std::max(part, (size_t)dense_chunks(sz[b]) * (size_t)std::max<int64_t>(sz[b], 1));
  }
  CTX_TRY(dalloc(&ctx->dn_part, 2 * part));
  ctx->dn_part_half = part;
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  for (int b = 0; b < 4; ++b) {
    ctx->dn_set[b] = true;
    ctx->dnR_set[b] = false;
  }
  ctx->dense = true;
  ctx->have_spec = true;
  return PEEC_OK;
}

// The dense retarded operator (iter_solver_QS_S_type.jl:39-59, QS_Rcc_FW == 2): the
// centre distances of the blocks (Lp_data[:Rx], [:Ry], [:Rz], P_data[:R_cc]; real,
// column-major, zero on the diagonal). Each frequency's blocks are the dense blocks times
// exp(-j beta R), formed on the device by peec_set_dense_rcc_frequency.
static int peec_set_dense_rcc_body(peec_ctx* ctx, const double* Rx, const double* Ry,
                                   const double* Rz, const double* Rcc) {
  if (!ctx) return badarg("peec_set_dense_rcc");
  if (!ctx->dense) return bad(ctx, PEEC_ERR_STATE, "no dense operator (peec_set_dense)");
  if (!Rx && !Ry && !Rz && !Rcc) {  // back to the quasi-static blocks
    drop_graphs(ctx);
    ctx->dense_rcc = ctx->dense_rcc_ready = false;
    return PEEC_OK;
  }
  const int64_t sz[4] = {ctx->mx, ctx->my, ctx->mz, ctx->ns};
  const double* src[4] = {Rx, Ry, Rz, Rcc};
  for (int b = 0; b < 4; ++b) {
    if (sz[b] > 0 && !src[b]) return bad(ctx, PEEC_ERR_BADARG, "peec_set_dense_rcc: missing block");
    for (int64_t i = 0; i < sz[b]; ++i)
      if (src[b][i * sz[b] + i] != 0.0)
        return bad(ctx, PEEC_ERR_BADARG, "peec_set_dense_rcc: distances must be zero on the diagonal");
  }
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  drop_graphs(ctx);
  ctx->dense_rcc = ctx->dense_rcc_ready = false;
  size_t part = 1;
  for (int b = 0; b < 4; ++b) {
    const int64_t ld = ctx->dn_ld[b];
    const size_t cnt = (size_t)ld * (size_t)sz[b];
    CTX_TRY(dalloc(&ctx->dnR[b], cnt));
    CTX_TRY(dalloc(&ctx->dnc64[b], cnt));
    CTX_TRY(dalloc(&ctx->dnc32[b], cnt));
    if (cnt) {
      PEEC_CUDA_TRY(cudaMemsetAsync(ctx->dnR[b], 0, sizeof(double) * cnt, ctx->st));
      PEEC_CUDA_TRY(cudaMemcpy2DAsync(ctx->dnR[b], sizeof(double) * ld, src[b],
                                      sizeof(double) * sz[b], sizeof(double) * sz[b], sz[b],
                                      cudaMemcpyHostToDevice, ctx->st));
    }
    // the scratch serves the real products too (a later peec_set_dense drops the phases)
    part = std::max({part, (size_t)dense_part_c(sz[b]),
                     (size_t)dense_chunks(sz[b]) * (size_t)std::max<int64_t>(sz[b], 1)});
  }
  part = std::max(part, (size_t)1);
  CTX_TRY(dalloc(&ctx->dn_part, 2 * part));
  ctx->dn_part_half = part;
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  for (int b = 0; b < 4; ++b) ctx->dnR_set[b] = true;
  ctx->dense_rcc = true;
  return PEEC_OK;
}

// the retarded blocks at beta = 2 pi f sqrt(eps0 mu0) (f in Hz): formed in place, so the
// captured graphs of the context stay valid. A context whose distances are on the device
// but which was switched back to the quasi-static blocks (peec_set_dense_rcc with NULLs)
// returns to the retarded operator here.
static int peec_set_dense_rcc_frequency_body(peec_ctx* ctx, double beta) {
  if (!ctx) return badarg("peec_set_dense_rcc_frequency");
  if (!ctx->dense_rcc) {
    if (!ctx->dense || !ctx->dnR_set[0] || !ctx->dnR_set[1] || !ctx->dnR_set[2] || !ctx->dnR_set[3])
      return bad(ctx, PEEC_ERR_STATE, "no dense distances (peec_set_dense_rcc)");
    drop_graphs(ctx);
    ctx->dense_rcc = true;
    ctx->dense_rcc_ready = false;
  }
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t sz[4] = {ctx->mx, ctx->my, ctx->mz, ctx->ns};
  for (int b = 0; b < 4; ++b) {
    const size_t cnt = (size_t)ctx->dn_ld[b] * (size_t)sz[b];
    if (cnt) dense_phase(ctx->dn64[b], ctx->dnR[b], cnt, beta, ctx->dnc64[b], ctx->dnc32[b], ctx->st);
  }
  ctx->launches += 4;
  PEEC_CUDA_TRY(cudaGetLastError());
  ctx->dense_rcc_ready = true;
  return PEEC_OK;
}

// The dense RIS matrices filled on the device (sharedRis/calcola_Lp.jl, calcola_P.jl)
// from the bodies' vertex coordinates, in place of peec_set_dense (+ peec_set_pdiag, and
// peec_set_dense_rcc with distances): vol_coords (m x 24, row-major: volumi[:coordinate]),
// vol_S (m, the cross-sections volumi[:S]), vol_centres (m x 3, volumi[:centri], read when
// distances); surf_ends (ns x 12, superfici["estremi_celle"]), surf_S (ns, superfici["S"]),
// surf_centres (ns x 3, superfici["centri"]). Either group may be NULL (its blocks are left
// as they are). *nonfinite (if given) gets the count of non-finite matrix entries.
static int peec_ris_fill_body(peec_ctx* ctx, const double* vol_coords, const double* vol_S,
                              const double* vol_centres, double escal_Lp, const double* surf_ends,
                              const double* surf_S, const double* surf_centres, double escal_P,
                              int distances, int64_t* nonfinite) {
  NvtxRange nvtx_range_("peec_ris_fill");
  if (!ctx) return badarg("peec_ris_fill");
  if (!ctx->have_topo || ctx->lattice)
    return bad(ctx, PEEC_ERR_STATE, "peec_ris_fill: needs the topology of peec_set_incidence");
  const bool vol = vol_coords != nullptr, surf = surf_ends != nullptr;
  if (!vol && !surf) return bad(ctx, PEEC_ERR_BADARG, "peec_ris_fill: no volumes and no surfaces");
  if ((vol && ctx->m > 0 && (!vol_S || (distances && !vol_centres))) ||
      (surf && ctx->ns > 0 && (!surf_S || (distances && !surf_centres))))
    return bad(ctx, PEEC_ERR_BADARG, "peec_ris_fill: missing cross-sections, areas or centres");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  drop_graphs(ctx);
  ctx->dense = false;
  ctx->dense_rcc = ctx->dense_rcc_ready = false;
  const int64_t sz[4] = {ctx->mx, ctx->my, ctx->mz, ctx->ns};
  const int64_t off[3] = {0, ctx->mx, ctx->mx + ctx->my};
  const size_t bb = ris_box_bytes();
  double *d_geom = nullptr, *d_S = nullptr, *d_ctr = nullptr, *d_self = nullptr;
  unsigned char* d_box = nullptr;
  int* d_nrm = nullptr;
  int* d_bad = nullptr;
  auto release = [&] {
    for (void* p : {(void*)d_geom, (void*)d_S, (void*)d_ctr, (void*)d_self, (void*)d_box,
                    (void*)d_nrm, (void*)d_bad})
      if (p) cudaFree(p);
  };
  int rc = PEEC_OK;
  auto put = [&](double** d, const double* h, size_t cnt) -> int {
    int r = dalloc(d, cnt);
    if (r) return r;
    if (cnt) PEEC_CUDA_TRY(cudaMemcpyAsync(*d, h, cnt * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
    return PEEC_OK;
  };
  auto block = [&](int b) -> int {
    const int64_t ld = dense_ld(sz[b]);
    ctx->dn_ld[b] = ld;
    const size_t cnt = (size_t)ld * (size_t)sz[b];
    int r = dalloc(&ctx->dn64[b], cnt);
    if (!r) r = dalloc(&ctx->dn32[b], cnt);
    if (r) return r;
    if (cnt) PEEC_CUDA_TRY(cudaMemsetAsync(ctx->dn64[b], 0, sizeof(double) * cnt, ctx->st));
    if (distances) {
      r = dalloc(&ctx->dnR[b], cnt);
      if (!r) r = dalloc(&ctx->dnc64[b], cnt);
      if (!r) r = dalloc(&ctx->dnc32[b], cnt);
      if (r) return r;
      if (cnt) PEEC_CUDA_TRY(cudaMemsetAsync(ctx->dnR[b], 0, sizeof(double) * cnt, ctx->st));
    }
    return PEEC_OK;
  };
  rc = [&]() -> int {
    if ((rc = dalloc(&d_bad, 1))) return rc;
    PEEC_CUDA_TRY(cudaMemsetAsync(d_bad, 0, sizeof(int), ctx->st));
    if (vol) {
      const int64_t m = ctx->m;
      if ((rc = put(&d_geom, vol_coords, (size_t)m * 24)) || (rc = put(&d_S, vol_S, (size_t)m)) ||
          (distances && (rc = put(&d_ctr, vol_centres, (size_t)m * 3))) ||
          (rc = dalloc(&d_self, (size_t)m)) || (rc = dalloc(&d_box, (size_t)m * bb)))
        return rc;
      if ((rc = ris_prep_gpu(0, d_geom, m, ctx->mx, ctx->my, d_box, d_self, nullptr, ctx->st))) return rc;
      const void* bx[3];
      const double *bS[3], *bself[3];
      double* bM[3];
      for (int b = 0; b < 3; ++b) {
        if ((rc = block(b))) return rc;
        bx[b] = d_box + (size_t)off[b] * bb;
        bS[b] = d_S + off[b];
        bself[b] = d_self + off[b];
        bM[b] = ctx->dn64[b];
      }
      // the three blocks in one launch
      if ((rc = ris_pairs_gpu(0, 3, bx, nullptr, bS, bself, sz, escal_Lp, bM, ctx->dn_ld, d_bad,
                              ctx->st)))
        return rc;
      for (int b = 0; b < 3 && !rc; ++b) {
        if (distances)
          rc = ris_dist_gpu(d_ctr + 3 * off[b], sz[b], ctx->dnR[b], ctx->dn_ld[b], ctx->st);
        if (!rc && sz[b])
          dense_round(ctx->dn64[b], (size_t)ctx->dn_ld[b] * sz[b], ctx->dn32[b], ctx->st);
        ctx->dn_set[b] = !rc;
        ctx->dnR_set[b] = !rc && distances;
      }
      if (rc) return rc;
    }
    if (surf) {
      const int64_t ns = ctx->ns;
      if ((rc = put(&d_geom, surf_ends, (size_t)ns * 12)) || (rc = put(&d_S, surf_S, (size_t)ns)) ||
          (distances && (rc = put(&d_ctr, surf_centres, (size_t)ns * 3))) ||
          (rc = dalloc(&d_nrm, (size_t)ns)) || (rc = dalloc(&d_box, (size_t)ns * bb)))
        return rc;
      if ((rc = ris_prep_gpu(1, d_geom, ns, 0, 0, d_box, nullptr, d_nrm, ctx->st))) return rc;
      if ((rc = block(3))) return rc;
      const void* bx[1] = {d_box};
      const double* bS[1] = {d_S};
      double* bM[1] = {ctx->dn64[3]};
      rc = ris_pairs_gpu(1, 1, bx, d_nrm, bS, nullptr, &sz[3], escal_P, bM, &ctx->dn_ld[3], d_bad,
                         ctx->st);
      if (!rc && distances) rc = ris_dist_gpu(d_ctr, ns, ctx->dnR[3], ctx->dn_ld[3], ctx->st);
      if (!rc && ns) dense_round(ctx->dn64[3], (size_t)ctx->dn_ld[3] * ns, ctx->dn32[3], ctx->st);
      if (!rc) rc = dalloc(&ctx->invP, (size_t)ns);
      if (!rc) rc = inv_diag_gpu(ctx->dn64[3], ctx->dn_ld[3], ns, ctx->invP, ctx->st);
      ctx->dn_set[3] = !rc;
      ctx->dnR_set[3] = !rc && distances;
      if (rc) return rc;
      ctx->have_pdiag = true;
    }
    size_t part = 1;
    for (int b = 0; b < 4; ++b) {
      part = std::max(part, (size_t)dense_chunks(sz[b]) * (size_t)std::max<int64_t>(sz[b], 1));
      if (distances) part = std::max(part, (size_t)dense_part_c(sz[b]));
    }
    if ((rc = dalloc(&ctx->dn_part, 2 * part))) return rc;
    ctx->dn_part_half = part;
    int hbad = 0;
    PEEC_CUDA_TRY(cudaMemcpyAsync(&hbad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
    if (nonfinite) *nonfinite = hbad;
    return PEEC_OK;
  }();
  release();
  if (rc) return rc;
  ctx->dense = ctx->dn_set[0] && ctx->dn_set[1] && ctx->dn_set[2] && ctx->dn_set[3];
  ctx->have_spec = ctx->dense;
  ctx->dense_rcc = ctx->dense && ctx->dnR_set[0] && ctx->dnR_set[1] && ctx->dnR_set[2] &&
                   ctx->dnR_set[3];
  return PEEC_OK;
}

// One dense block back to the host (column-major, n x n): what 0 the matrix, 1 its centre
// distances, 2 its diagonal (n values). block 0..2: Lp_x, Lp_y, Lp_z; 3: P.
static int peec_dense_get_body(peec_ctx* ctx, int block, int what, double* out) {
  if (!ctx) return badarg("peec_dense_get");
  if (block < 0 || block > 3 || what < 0 || what > 2 || !out)
    return bad(ctx, PEEC_ERR_BADARG, "peec_dense_get: block 0..3, what 0..2, out required");
  if (!ctx->dn_set[block] || (what == 1 && !ctx->dnR_set[block]))
    return bad(ctx, PEEC_ERR_STATE, "peec_dense_get: block not set");
  const int64_t n = block < 3 ? (block == 0 ? ctx->mx : (block == 1 ? ctx->my : ctx->mz)) : ctx->ns;
  if (n == 0) return PEEC_OK;
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t ld = ctx->dn_ld[block];
  const double* src = what == 1 ? ctx->dnR[block] : ctx->dn64[block];
  if (what == 2)
    PEEC_CUDA_TRY(cudaMemcpy2DAsync(out, sizeof(double), src, sizeof(double) * (ld + 1),
                                    sizeof(double), n, cudaMemcpyDeviceToHost, ctx->st));
  else
    PEEC_CUDA_TRY(cudaMemcpy2DAsync(out, sizeof(double) * n, src, sizeof(double) * ld,
                                    sizeof(double) * n, n, cudaMemcpyDeviceToHost, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return PEEC_OK;
}

static int peec_set_pdiag_body(peec_ctx* ctx, const double* diagP) {
  drop_graphs(ctx);
  if (!ctx || !diagP) return badarg("peec_set_pdiag");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  std::vector<double> inv(ctx->ns);
  for (int64_t s = 0; s < ctx->ns; ++s) inv[s] = 1.0 / diagP[s];
  CTX_TRY(upload(&ctx->invP, inv, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->have_pdiag = true;
  return PEEC_OK;
}

// The FP32 z-pass autotuner. For this context's grids it times every eligible form of the
// face families' z pass and every form x radix plan of the edge families' z pass (one
// warm-up launch, then the mean of three, CUDA events on the context stream) and keeps the
// fastest; choices are cached process-wide by device and grids, so clones and later
// contexts of the same lattice reuse them. The candidates run on the context's FP32 family
// buffers, which every operator application rewrites from its input before the z passes.
struct ZChoice {
  int face = 0, edge = 0, plan = 0;
  double fms[3] = {-1, -1, -1};
  double ems[6] = {-1, -1, -1, -1, -1, -1};
};
static std::mutex g_tune_mu;
static std::map<std::vector<int>, ZChoice> g_tune;
static int check_solve_errors(peec_ctx* ctx);

static int tune_zpass(peec_ctx* ctx) {
  ctx->zt.err = ctx->zerr;
  ctx->zt.nsm = ctx->nsm;
  std::vector<int> key{ctx->dev};
  for (const auto& F : ctx->fam) {
    key.push_back(F.active ? 1 : 0);
    for (int k = 0; k < 3; ++k) key.push_back(F.L[k]);
    key.push_back(F.dims[2]);
  }
  auto apply = [&](const ZChoice& c) {
    ctx->zt.face = c.face;
    ctx->zt.edge = c.edge;
    ctx->zt.edge_plan = c.plan;
    std::memcpy(ctx->zface_ms, c.fms, sizeof(c.fms));
    std::memcpy(ctx->zedge_ms, c.ems, sizeof(c.ems));
  };
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return apply(it->second), PEEC_OK;
  }
  for (const auto& F : ctx->fam)
    if (F.active && F.T[1])
      PEEC_CUDA_TRY(cudaMemsetAsync(F.T[1], 0, (size_t)F.L[0] * F.L[1] * F.dims[2] * sizeof(c32),
                                    ctx->st));
  const void* ph[6] = {ctx->ph64[0], ctx->ph64[1], ctx->ph64[2],
                       ctx->ph32[0], ctx->ph32[1], ctx->ph32[2]};
  auto timed = [&](const ZTune& z, int which, double* ms) -> int {
    CTX_TRY(zpass_f32(ctx->fam, 6, ctx->spec, ph, ctx->tw32, ctx->twmax, z, which, ctx->st));
    PEEC_CUDA_TRY(cudaEventRecord(ctx->ev[0], ctx->st));
    for (int i = 0; i < 3; ++i)
      CTX_TRY(zpass_f32(ctx->fam, 6, ctx->spec, ph, ctx->tw32, ctx->twmax, z, which, ctx->st));
    PEEC_CUDA_TRY(cudaEventRecord(ctx->ev[1], ctx->st));
    PEEC_CUDA_TRY(cudaEventSynchronize(ctx->ev[1]));
    float t = 0;
    PEEC_CUDA_TRY(cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
    *ms = t / 3.0;
    return PEEC_OK;
  };
  ZChoice c;
  const bool faces = ctx->fam[0].active && ctx->fam[1].active && ctx->fam[2].active;
  bool edges = false;
  for (int f = 3; f < 6; ++f) edges |= ctx->fam[f].active;
  ZTune z = ctx->zt;
  if (faces) {
    const int nform = zpass_yz_faces(ctx->fam, 6) ? 3 : 1;
    for (int form = 0; form < nform; ++form) {
      z.face = form;
      CTX_TRY(timed(z, 0, &c.fms[form]));
      if (c.fms[form] < c.fms[c.face]) c.face = form;
    }
  }
  if (edges) {
    const int nform = zpass_yz_edges(ctx->fam, 6) ? 3 : 1;
    double best = -1;
    for (int plan = 0; plan < 2; ++plan) {
      for (int form = 0; form < nform; ++form) {
        z.edge = form;
        z.edge_plan = plan;
        double& ms = c.ems[plan * 3 + form];
        CTX_TRY(timed(z, 1, &ms));
        if (best < 0 || ms < best) {
          best = ms;
          c.edge = form;
          c.plan = plan;
        }
      }
    }
  }
  CTX_TRY(check_solve_errors(ctx));
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[key] = c;
  }
  apply(c);
  return PEEC_OK;
}

// spectra from device rows (rows in the order Lpx, Lpy, Lpz, p12, p34, p56, p1234,
// p1256, p3456). Spectrum i uses row srow[i]: P blocks 00, 11, 22 (symmetric), 01, 02, 12
// (cross: output family f, input family g), then the three Lp blocks.
static int build_spectrum_set(peec_ctx* ctx, Spectrum* dst, double* const d_rows[9]) {
  static const int srow[9] = {3, 4, 5, 6, 7, 8, 0, 1, 2};
  static const int fout[9] = {0, 1, 2, 0, 0, 1, 3, 4, 5};
  static const int fin[9] = {0, 1, 2, 1, 2, 2, 3, 4, 5};
  static const int sdim[9][3] = {{1, 1, 1}, {1, 1, 1}, {1, 1, 1}, {2, 2, 1}, {1, 2, 2},
                                 {2, 1, 2}, {1, 1, 1}, {1, 1, 1}, {1, 1, 1}};
  static const int odim[9][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, -1, 0}, {0, -1, 1},
                                 {-1, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int i = 0; i < 9; ++i) {
    if (!ctx->fam[fout[i]].active || !ctx->fam[fin[i]].active) continue;
    if (!d_rows[srow[i]]) return bad(ctx, PEEC_ERR_BADARG, "missing generating row");
    const bool sym = i < 3 || i >= 6;
    CTX_TRY(spectrum_build(dst[i], d_rows[srow[i]], ctx->row_dims[srow[i]],
                           ctx->fam[fout[i]].dims, ctx->fam[fin[i]].dims, sdim[i], odim[i],
                           sym ? 1 : 0, ctx->tw64, ctx->twmax, ctx->st));
    ctx->launches += 6;
  }
  return PEEC_OK;
}

static int build_spectra(peec_ctx* ctx, double* const d_rows[9]) {
  drop_graphs(ctx);
  ctx->cc_prec = -1;
  ctx->rcc = false;
  ctx->dense = false;  // the circulant operator replaces dense matrices set before
  CTX_TRY(build_spectrum_set(ctx, ctx->spec, d_rows));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->have_spec = true;
  CTX_TRY(tune_zpass(ctx));
  return PEEC_OK;
}

static int peec_set_rows_body(peec_ctx* ctx, const double* const rows[9]) {
  NvtxRange nvtx_range_("peec_set_rows");
  if (!ctx || !rows) return badarg("peec_set_rows");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  if (!ctx->lattice) return bad(ctx, PEEC_ERR_STATE, "no voxel lattice (peec_set_incidence topology)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  double* d_rows[9] = {};
  int rc = PEEC_OK;
  for (int i = 0; i < 9 && rc == PEEC_OK; ++i) {
    const size_t len = (size_t)ctx->row_dims[i][0] * ctx->row_dims[i][1] * ctx->row_dims[i][2];
    if (len == 0 || !rows[i]) continue;
    if (cudaMalloc(&d_rows[i], len * sizeof(double)) != cudaSuccess) {
      rc = bad(ctx, PEEC_ERR_OOM, "row upload allocation");
      break;
    }
    cudaMemcpyAsync(d_rows[i], rows[i], len * sizeof(double), cudaMemcpyHostToDevice, ctx->st);
  }
  if (rc == PEEC_OK) rc = build_spectra(ctx, d_rows);
  cudaStreamSynchronize(ctx->st);
  for (auto p : d_rows)
    if (p) cudaFree(p);
  return rc;
}

static int peec_fill_body(peec_ctx* ctx, const double origin[3], double sx, double sy, double sz,
                         double escal_Lp, double escal_P, double* const rows_out[9]) {
  NvtxRange nvtx_range_("peec_fill");
  if (!ctx || !origin) return badarg("peec_fill");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  if (!ctx->lattice) return bad(ctx, PEEC_ERR_STATE, "no voxel lattice (peec_set_incidence topology)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  double* d_rows[9] = {};
  int64_t len[9];
  int rc = PEEC_OK;
  int* d_bad = nullptr;
  PEEC_CUDA_TRY(cudaMalloc(&d_bad, sizeof(int)));
  PEEC_CUDA_TRY(cudaMemsetAsync(d_bad, 0, sizeof(int), ctx->st));
  for (int i = 0; i < 9; ++i) {
    len[i] = (int64_t)ctx->row_dims[i][0] * ctx->row_dims[i][1] * ctx->row_dims[i][2];
    if (len[i] > 0 && cudaMalloc(&d_rows[i], len[i] * sizeof(double)) != cudaSuccess) {
      rc = bad(ctx, PEEC_ERR_OOM, "row allocation");
      break;
    }
  }
  if (rc == PEEC_OK) {
    rc = fill_rows_gpu(origin, sx, sy, sz, escal_Lp, escal_P, ctx->Nx, ctx->Ny, ctx->Nz, d_rows,
                       len, d_bad, ctx->st);
    ctx->launches += 9;
    if (rc) ctx->err = g_err;
  }
  int hbad = 0;
  if (rc == PEEC_OK) {
    cudaMemcpyAsync(&hbad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
    if (cudaStreamSynchronize(ctx->st) != cudaSuccess)
      rc = fail_cuda(cudaGetLastError(), "fill", __FILE__, __LINE__);
    else if (hbad)
      rc = bad(ctx, PEEC_ERR_UNSUPPORTED,
               "fill: a row entry is not finite (degenerate cell sizes?)");
  }
  if (rc == PEEC_OK && rows_out) {
    for (int i = 0; i < 9; ++i)
      if (rows_out[i] && d_rows[i])
        cudaMemcpyAsync(rows_out[i], d_rows[i], len[i] * sizeof(double), cudaMemcpyDeviceToHost,
                        ctx->st);
  }
  if (rc == PEEC_OK) rc = build_spectra(ctx, d_rows);
  cudaStreamSynchronize(ctx->st);
  for (auto p : d_rows)
    if (p) cudaFree(p);
  cudaFree(d_bad);
  return rc;
}

// ------------------------------------------------------------------------------------
// retarded (Rcc) operator
// ------------------------------------------------------------------------------------

static int rcc_alloc_rows(peec_ctx* ctx, int64_t len[9]) {
  for (int i = 0; i < 9; ++i) {
    len[i] = (int64_t)ctx->row_dims[i][0] * ctx->row_dims[i][1] * ctx->row_dims[i][2];
    if (len[i] > 0 && !ctx->rcc_qs[i])
      if (cudaMalloc(&ctx->rcc_qs[i], len[i] * sizeof(double)) != cudaSuccess)
        return bad(ctx, PEEC_ERR_OOM, "Rcc row allocation");
  }
  return PEEC_OK;
}

static void rcc_geometry(peec_ctx* ctx, const double origin[3], double sx, double sy, double sz) {
  for (int q = 0; q < 3; ++q) ctx->rcc_origin[q] = origin[q];
  ctx->rcc_s[0] = sx;
  ctx->rcc_s[1] = sy;
  ctx->rcc_s[2] = sz;
  ctx->have_rcc_rows = true;
  ctx->rcc_freq = -1.0;
}

static int peec_fill_rcc_body(peec_ctx* ctx, const double origin[3], double sx, double sy,
                              double sz, double escal_Lp, double escal_P,
                              double* const rows_out[9]) {
  NvtxRange nvtx_range_("peec_fill_rcc");
  if (!ctx || !origin) return badarg("peec_fill_rcc");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  if (!ctx->lattice) return bad(ctx, PEEC_ERR_STATE, "no voxel lattice (peec_set_incidence topology)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  int64_t len[9];
  ctx->have_rcc_rows = false;
  CTX_TRY(rcc_alloc_rows(ctx, len));
  int* d_bad = nullptr;
  PEEC_CUDA_TRY(cudaMalloc(&d_bad, sizeof(int)));
  cudaMemsetAsync(d_bad, 0, sizeof(int), ctx->st);
  int rc = fill_rows_rcc_gpu(origin, sx, sy, sz, escal_Lp, escal_P, ctx->Nx, ctx->Ny, ctx->Nz,
                             ctx->rcc_qs, len, d_bad, ctx->st);
  ctx->launches += 9;
  if (rc) ctx->err = g_err;
  int hbad = 0;
  if (rc == PEEC_OK) {
    cudaMemcpyAsync(&hbad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
    if (cudaStreamSynchronize(ctx->st) != cudaSuccess)
      rc = fail_cuda(cudaGetLastError(), "fill_rcc", __FILE__, __LINE__);
    else if (hbad & 2)
      rc = bad(ctx, PEEC_ERR_UNSUPPORTED,
               "fill_rcc: an Lp entry falls in the orthogonal surface-surface case of the Rcc "
               "dispatcher, which the reference cannot evaluate (compute_Lp_Voxels_QS.jl:330-352)");
    else if (hbad)
      rc = bad(ctx, PEEC_ERR_UNSUPPORTED,
               "fill_rcc: a row entry is not finite (degenerate cell sizes?)");
  }
  cudaFree(d_bad);
  if (rc != PEEC_OK) return rc;
  if (rows_out)
    for (int i = 0; i < 9; ++i)
      if (rows_out[i] && len[i] > 0)
        cudaMemcpyAsync(rows_out[i], ctx->rcc_qs[i], len[i] * sizeof(double),
                        cudaMemcpyDeviceToHost, ctx->st);
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  rcc_geometry(ctx, origin, sx, sy, sz);
  return PEEC_OK;
}

static int peec_set_rows_rcc_body(peec_ctx* ctx, const double* const rows[9],
                                  const double origin[3], double sx, double sy, double sz) {
  NvtxRange nvtx_range_("peec_set_rows_rcc");
  if (!ctx || !rows || !origin) return badarg("peec_set_rows_rcc");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  if (!ctx->lattice) return bad(ctx, PEEC_ERR_STATE, "no voxel lattice (peec_set_incidence topology)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  int64_t len[9];
  ctx->have_rcc_rows = false;
  CTX_TRY(rcc_alloc_rows(ctx, len));
  for (int i = 0; i < 9; ++i) {
    if (len[i] == 0) continue;
    if (!rows[i]) return bad(ctx, PEEC_ERR_BADARG, "missing Rcc generating row");
    cudaMemcpyAsync(ctx->rcc_qs[i], rows[i], len[i] * sizeof(double), cudaMemcpyHostToDevice,
                    ctx->st);
  }
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  rcc_geometry(ctx, origin, sx, sy, sz);
  return PEEC_OK;
}

// The spectra of the Rcc rows at freq_hz: row * exp(-i beta R) with
// beta = 2 pi f sqrt(eps0 mu0) (build_row_vox_Rcc.jl:1-11), split into real and
// imaginary rows, each embedded and transformed like a QS row
// (compute_Circulant_Lp_Rcc.jl, compute_Circulant_P_sup_Rcc.jl). The operator is linear
// in its rows, so K x = K_re x + i K_im x with both halves real-row circulant operators.
static int peec_set_rcc_frequency_body(peec_ctx* ctx, double freq_hz) {
  NvtxRange nvtx_range_("peec_set_rcc_frequency");
  if (!ctx) return badarg("peec_set_rcc_frequency");
  if (!ctx->have_rcc_rows) return bad(ctx, PEEC_ERR_STATE, "Rcc rows not set");
  if (!(freq_hz >= 0.0) || !std::isfinite(freq_hz))
    return bad(ctx, PEEC_ERR_BADARG, "frequency must be finite and >= 0");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  if (ctx->rcc && ctx->rcc_freq == freq_hz) return PEEC_OK;
  const double pi = 3.141592653589793;
  const double mu0 = 4 * pi * 1e-7;
  const double eps0 = 8.854187816997944e-12;
  const double beta = 2 * pi * freq_hz * std::sqrt(eps0 * mu0);
  int64_t len[9];
  double* re[9] = {};
  double* im[9] = {};
  int rc = PEEC_OK;
  for (int i = 0; i < 9 && rc == PEEC_OK; ++i) {
    len[i] = (int64_t)ctx->row_dims[i][0] * ctx->row_dims[i][1] * ctx->row_dims[i][2];
    if (len[i] == 0) continue;
    if (cudaMallocAsync(&re[i], len[i] * sizeof(double), ctx->st) != cudaSuccess ||
        cudaMallocAsync(&im[i], len[i] * sizeof(double), ctx->st) != cudaSuccess)
      rc = bad(ctx, PEEC_ERR_OOM, "Rcc phased rows");
  }
  drop_graphs(ctx);
  ctx->cc_prec = -1;
  ctx->rcc = false;
  if (rc == PEEC_OK) {
    rc = rcc_rows_gpu(ctx->rcc_origin, ctx->rcc_s[0], ctx->rcc_s[1], ctx->rcc_s[2], ctx->Nx,
                      ctx->Ny, ctx->Nz, beta, ctx->rcc_qs, re, im, len, ctx->st);
    ctx->launches += 9;
    if (rc) ctx->err = g_err;
  }
  if (rc == PEEC_OK) rc = build_spectrum_set(ctx, ctx->spec, re);
  if (rc == PEEC_OK) rc = build_spectrum_set(ctx, ctx->spec_im, im);
  for (int i = 0; i < 9; ++i) {
    if (re[i]) cudaFreeAsync(re[i], ctx->st);
    if (im[i]) cudaFreeAsync(im[i], ctx->st);
  }
  const cudaError_t e = cudaStreamSynchronize(ctx->st);
  if (rc != PEEC_OK) return rc;
  if (e != cudaSuccess) return fail_cuda(e, "Rcc spectra", __FILE__, __LINE__);
  const bool tuned = ctx->have_spec && !ctx->dense;
  ctx->have_spec = true;
  ctx->dense = false;
  ctx->rcc = true;
  ctx->rcc_freq = freq_hz;
  if (!tuned) CTX_TRY(tune_zpass(ctx));
  return PEEC_OK;
}

// ------------------------------------------------------------------------------------
// frequency state
// ------------------------------------------------------------------------------------

// Splits a CSR triangular factor into off-diagonal CSR + inverse diagonal and
// computes dependency levels (lower: increasing, upper: decreasing row order).
static int make_tri(peec_ctx* ctx, LevelTri& T, int64_t n, const int64_t* ptr, const int64_t* col,
                    const double* val, bool lower) {
  free_tri(T);
  std::vector<int32_t> p(n + 1, 0), c;
  std::vector<c64> v, dinv(n);
  c.reserve(ptr[n]);
  v.reserve(ptr[n]);
  std::vector<int> level(n, 0);
  for (int64_t r = 0; r < n; ++r) {
    cd diag(0.0, 0.0);
    for (int64_t q = ptr[r]; q < ptr[r + 1]; ++q) {
      const int64_t j = col[q];
      const cd x(val[2 * q], val[2 * q + 1]);
      if (j == r) {
        diag = x;
      } else {
        if ((lower && j > r) || (!lower && j < r))
          return bad(ctx, PEEC_ERR_BADARG, "triangular factor has entries on the wrong side");
        if (j < 0 || j >= n) return bad(ctx, PEEC_ERR_BADARG, "triangular factor column out of range");
        c.push_back((int32_t)j);
        v.push_back(mk<double>(x.real(), x.imag()));
      }
    }
    if (diag == cd(0.0, 0.0)) return bad(ctx, PEEC_ERR_BADARG, "zero pivot in triangular factor");
    const cd di = 1.0 / diag;
    dinv[r] = mk<double>(di.real(), di.imag());
    p[r + 1] = (int32_t)c.size();
  }
  // levels
  int maxl = 0;
  if (lower) {
    for (int64_t r = 0; r < n; ++r) {
      int l = 0;
      for (int32_t q = p[r]; q < p[r + 1]; ++q) l = std::max(l, level[c[q]] + 1);
      level[r] = l;
      maxl = std::max(maxl, l);
    }
  } else {
    for (int64_t r = n - 1; r >= 0; --r) {
      int l = 0;
      for (int32_t q = p[r]; q < p[r + 1]; ++q) l = std::max(l, level[c[q]] + 1);
      level[r] = l;
      maxl = std::max(maxl, l);
    }
  }
  std::vector<int> cnt(maxl + 2, 0);
  for (int64_t r = 0; r < n; ++r) cnt[level[r] + 1]++;
  for (int l = 0; l <= maxl; ++l) cnt[l + 1] += cnt[l];
  std::vector<int32_t> rows(n);
  std::vector<int> fillp(cnt.begin(), cnt.end() - 1);
  for (int64_t r = 0; r < n; ++r) rows[fillp[level[r]]++] = (int32_t)r;
  T.lvl_off.assign(cnt.begin(), cnt.end());
  T.rows = std::move(rows);
  CTX_TRY(upload(&T.ptr, p, ctx->st));
  CTX_TRY(upload(&T.col, c, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));  // the uploads read p and c
  T.hptr = std::move(p);
  T.hcol = std::move(c);
  CTX_TRY(upload(&T.val, v, ctx->st));
  CTX_TRY(upload(&T.dinv, dinv, ctx->st));
  // ready flags start below every epoch the solve will use (epochs start at 1)
  CTX_TRY(dalloc(&T.flag, (size_t)n));
  PEEC_CUDA_TRY(cudaMemsetAsync(T.flag, 0, sizeof(int32_t) * n, ctx->st));
  T.nflag = n;
  return PEEC_OK;
}

// Work split of the LU solves. The rows of L and U fall into connected components
// (rows linked by a factor entry); rows of different components never depend on one
// another. Components of at most comp_max rows are solved per warp (k_sptrsv_grp): those
// of at most 32 rows and SF_GRP_E entries packed into groups of at most 32 rows and
// SF_GRP_E entries, in order of their level depth (so that a group's levels are mostly
// full), larger ones one per group; the rows of components above comp_max (or too large
// for a warp's shared memory) go to the synchronisation-free global scheme.
static int build_solve_plan(peec_ctx* ctx, int64_t n) {
  const LevelTri &L = ctx->Lf, &U = ctx->Uf;
  // union-find over the factor entries
  std::vector<int32_t> parent(n);
  for (int64_t r = 0; r < n; ++r) parent[r] = (int32_t)r;
  auto find = [&](int32_t a) {
    while (parent[a] != a) {
      parent[a] = parent[parent[a]];
      a = parent[a];
    }
    return a;
  };
  for (const LevelTri* T : {&L, &U})
    for (int64_t r = 0; r < n; ++r)
      for (int32_t q = T->hptr[r]; q < T->hptr[r + 1]; ++q) {
        const int32_t a = find((int32_t)r), b = find(T->hcol[q]);
        if (a != b) parent[std::max(a, b)] = std::min(a, b);
      }
  std::vector<int32_t> comp(n), csize(n, 0), cent(n, 0), cdepth(n, 0);
  // per-row levels
  std::vector<int32_t> lvL(n), lvU(n);
  for (size_t l = 0; l + 1 < L.lvl_off.size(); ++l)
    for (int q = L.lvl_off[l]; q < L.lvl_off[l + 1]; ++q) lvL[L.rows[q]] = (int32_t)l;
  for (size_t l = 0; l + 1 < U.lvl_off.size(); ++l)
    for (int q = U.lvl_off[l]; q < U.lvl_off[l + 1]; ++q) lvU[U.rows[q]] = (int32_t)l;
  for (int64_t r = 0; r < n; ++r) {
    const int32_t c = comp[r] = find((int32_t)r);
    csize[c]++;
    cent[c] += (L.hptr[r + 1] - L.hptr[r]) + (U.hptr[r + 1] - U.hptr[r]);
    cdepth[c] = std::max(cdepth[c], lvL[r] + lvU[r] + 2);
  }
  // largest groups a warp's shared memory takes (a large component alone)
  const size_t smem_cap = 160 * 1024;
  std::vector<int32_t> big, small;
  for (int64_t r = 0; r < n; ++r) {
    if (comp[r] != r || csize[r] > ctx->comp_max) continue;
    if (csize[r] <= 32 && cent[r] <= SF_GRP_E) small.push_back((int32_t)r);
    else if (cent[r] < 32768 && grp_smem(csize[r], cent[r]) <= smem_cap) big.push_back((int32_t)r);
  }
  // large components, longest chains first; small ones by depth
  std::stable_sort(big.begin(), big.end(),
                   [&](int32_t a, int32_t b) { return cdepth[a] > cdepth[b]; });
  std::stable_sort(small.begin(), small.end(),
                   [&](int32_t a, int32_t b) { return cdepth[a] > cdepth[b]; });
  std::vector<int32_t> gidx(n, -1);  // component root -> group
  int ng = 0, rb = 0, eb = 0;
  for (int32_t c : big) {
    gidx[c] = ng++;
    rb = std::max(rb, csize[c]);
    eb = std::max(eb, cent[c]);
  }
  const int nbig = ng;
  {
    int rows = 0, ents = 0;
    for (int32_t c : small) {
      if (ng == nbig || rows + csize[c] > 32 || ents + cent[c] > SF_GRP_E) {
        ++ng;
        rows = ents = 0;
      }
      gidx[c] = ng - 1;
      rows += csize[c];
      ents += cent[c];
    }
  }
  // the groups' rows, in L-level order within each group
  std::vector<int32_t> goff(ng + 1, 0);
  for (int64_t r = 0; r < n; ++r)
    if (gidx[comp[r]] >= 0) goff[gidx[comp[r]] + 1]++;
  for (int g = 0; g < ng; ++g) goff[g + 1] += goff[g];
  std::vector<int32_t> rowsL(goff[ng]), fill(goff.begin(), goff.end() - 1);
  for (int64_t r = 0; r < n; ++r)
    if (gidx[comp[r]] >= 0) rowsL[fill[gidx[comp[r]]]++] = (int32_t)r;
  std::vector<int32_t> rowsU(rowsL), local(n, -1), seg, segoff(ng + 1, 0), nsegL(ng, 0);
  std::vector<GrpRow> grows(goff[ng]);
  std::vector<int16_t> uq(goff[ng]);
  for (int g = 0; g < ng; ++g) {
    const auto b0 = rowsL.begin() + goff[g], e0 = rowsL.begin() + goff[g + 1];
    std::stable_sort(b0, e0, [&](int32_t x, int32_t y) { return lvL[x] < lvL[y]; });
    for (int32_t q = goff[g]; q < goff[g + 1]; ++q) local[rowsL[q]] = q - goff[g];
    for (int32_t q = goff[g]; q < goff[g + 1]; ++q)
      if (q + 1 == goff[g + 1] || lvL[rowsL[q + 1]] != lvL[rowsL[q]]) seg.push_back(q + 1 - goff[g]);
    nsegL[g] = (int32_t)seg.size() - segoff[g];
    const auto bu = rowsU.begin() + goff[g], eu = rowsU.begin() + goff[g + 1];
    std::stable_sort(bu, eu, [&](int32_t x, int32_t y) { return lvU[x] < lvU[y]; });
    for (int32_t q = goff[g]; q < goff[g + 1]; ++q) {
      uq[q] = (int16_t)local[rowsU[q]];
      if (q + 1 == goff[g + 1] || lvU[rowsU[q + 1]] != lvU[rowsU[q]]) seg.push_back(q + 1 - goff[g]);
    }
    segoff[g + 1] = (int32_t)seg.size();
    int e = 0;
    for (int32_t q = goff[g]; q < goff[g + 1]; ++q) {
      const int32_t r = rowsL[q];
      GrpRow& gr = grows[q];
      gr.r = r;
      gr.pL = L.hptr[r];
      gr.pU = U.hptr[r];
      gr.j = ctx->h_gin.empty() ? r : ctx->h_gin[r];
      gr.nL = (int16_t)(L.hptr[r + 1] - L.hptr[r]);
      gr.nU = (int16_t)(U.hptr[r + 1] - U.hptr[r]);
      gr.eL = (int16_t)e;
      e += gr.nL;
      gr.eU = (int16_t)e;
      e += gr.nU;
    }
  }
  // entry columns as positions in the row's group
  std::vector<int16_t> lcolL(std::max<size_t>(L.hcol.size(), 1), -1),
      lcolU(std::max<size_t>(U.hcol.size(), 1), -1);
  for (const auto* T : {&L, &U}) {
    std::vector<int16_t>& lc = T == &L ? lcolL : lcolU;
    for (int64_t r = 0; r < n; ++r)
      if (local[r] >= 0)
        for (int32_t q = T->hptr[r]; q < T->hptr[r + 1]; ++q) lc[q] = (int16_t)local[T->hcol[q]];
  }
  if (ng == 0) {  // keep the arrays non-empty
    seg.push_back(0);
    rowsL.push_back(0);
    grows.push_back(GrpRow());
    uq.push_back(0);
    nsegL.push_back(0);
  }
  CTX_TRY(upload(&ctx->grp_goff, goff, ctx->st));
  CTX_TRY(upload(&ctx->grp_rows, grows, ctx->st));
  CTX_TRY(upload(&ctx->grp_uq, uq, ctx->st));
  CTX_TRY(upload(&ctx->grp_seg, seg, ctx->st));
  CTX_TRY(upload(&ctx->grp_segoff, segoff, ctx->st));
  CTX_TRY(upload(&ctx->grp_nsegL, nsegL, ctx->st));
  CTX_TRY(upload(&ctx->grp_lcolL, lcolL, ctx->st));
  CTX_TRY(upload(&ctx->grp_lcolU, lcolU, ctx->st));
  GrpPlan& P = ctx->grp;
  P.goff = ctx->grp_goff;
  P.rows = ctx->grp_rows;
  P.uq = ctx->grp_uq;
  P.seg = ctx->grp_seg;
  P.segoff = ctx->grp_segoff;
  P.nsegL = ctx->grp_nsegL;
  P.lcolL = ctx->grp_lcolL;
  P.lcolU = ctx->grp_lcolU;
  P.nbig = nbig;
  P.ngroups = ng;
  P.rb = rb;
  P.eb = eb;
  const size_t need = std::max(grp_smem(rb, eb), SF_GRP_WARPS * grp_smem(32, SF_GRP_E));
  if (sptrsv_grp_prepare(need)) return PEEC_ERR_CUDA;
  std::vector<int32_t> cidx(n, -1);
  for (int64_t r = 0; r < n; ++r) cidx[r] = gidx[comp[r]];
  // claim order of the global scheme: rows of the large components only
  std::vector<int32_t> ord;
  for (const LevelTri* T : {&L, &U}) {
    for (size_t l = 0; l + 1 < T->lvl_off.size(); ++l) {
      const size_t before = ord.size();
      for (int q = T->lvl_off[l]; q < T->lvl_off[l + 1]; ++q)
        if (cidx[comp[T->rows[q]]] < 0) ord.push_back(T->rows[q]);
      if (ord.size() != before)
        while (ord.size() % 32) ord.push_back(-1);
    }
    if (T == &L) ctx->sf_nL = (int)ord.size();
  }
  if (ord.size() > (size_t)INT32_MAX - 64) return bad(ctx, PEEC_ERR_UNSUPPORTED, "LU too large");
  ctx->sf_total = (int)ord.size();
  if (ord.empty()) ord.push_back(-1);
  CTX_TRY(upload(&ctx->sf_ord, ord, ctx->st));
  if (!ctx->sf_ctl) {
    CTX_TRY(dalloc(&ctx->sf_ctl, 4));
    PEEC_CUDA_TRY(cudaMemsetAsync(ctx->sf_ctl, 0, sizeof(int) * 4, ctx->st));
  }
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return PEEC_OK;
}

// Yle from COO to CSR with duplicates summed, as sparse() does
static int yle_csr(peec_ctx* ctx, int64_t n, int64_t yle_nnz, const int64_t* yle_row,
                   const int64_t* yle_col, const double* yle_val, std::vector<int32_t>& yp,
                   std::vector<int32_t>& yc, std::vector<c64>& yv) {
  yp.assign(n + 1, 0);
  yc.clear();
  yv.clear();
  {
    std::vector<std::vector<std::pair<int32_t, cd>>> rowsv(n);
    for (int64_t q = 0; q < yle_nnz; ++q) {
      if (yle_row[q] < 0 || yle_row[q] >= n || yle_col[q] < 0 || yle_col[q] >= n)
        return bad(ctx, PEEC_ERR_BADARG, "Yle index out of range");
      rowsv[yle_row[q]].push_back({(int32_t)yle_col[q], cd(yle_val[2 * q], yle_val[2 * q + 1])});
    }
    for (int64_t r = 0; r < n; ++r) {
      auto& rv = rowsv[r];
      std::sort(rv.begin(), rv.end(),
                [](const std::pair<int32_t, cd>& a, const std::pair<int32_t, cd>& b) {
                  return a.first < b.first;
                });
      for (size_t i = 0; i < rv.size(); ++i) {
        if (!yc.empty() && (int64_t)yp[r] < (int64_t)yc.size() && yc.back() == rv[i].first &&
            yc.size() > (size_t)yp[r]) {
          c64& t = yv.back();
          t.x += rv[i].second.real();
          t.y += rv[i].second.imag();
        } else {
          yc.push_back(rv[i].first);
          yv.push_back(mk<double>(rv[i].second.real(), rv[i].second.imag()));
        }
      }
      yp[r + 1] = (int32_t)yc.size();
    }
  }
  return PEEC_OK;
}

static int peec_set_frequency_body(peec_ctx* ctx, double w, const double* DZ, int64_t yle_nnz,
                                  const int64_t* yle_row, const int64_t* yle_col,
                                  const double* yle_val, const int64_t* L_ptr,
                                  const int64_t* L_col, const double* L_val,
                                  const int64_t* U_ptr, const int64_t* U_col,
                                  const double* U_val, const int64_t* perm_r,
                                  const int64_t* perm_c, const double* row_scale) {
  NvtxRange nvtx_range_("peec_set_frequency");
  drop_graphs(ctx);
  if (!ctx || !DZ || !L_ptr || !U_ptr || !perm_r || !perm_c) return badarg("peec_set_frequency");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t n = ctx->n, m = ctx->m;
  ctx->w = w;
  std::vector<c64> dz(m);
  for (int64_t e = 0; e < m; ++e) dz[e] = mk<double>(DZ[2 * e], DZ[2 * e + 1]);
  CTX_TRY(upload(&ctx->DZ, dz, ctx->st));
  // Yle COO -> CSR (duplicates summed, as sparse() does)
  std::vector<int32_t> yp, yc;
  std::vector<c64> yv;
  CTX_TRY(yle_csr(ctx, n, yle_nnz, yle_row, yle_col, yle_val, yp, yc, yv));
  CTX_TRY(upload(&ctx->yle_ptr, yp, ctx->st));
  CTX_TRY(upload(&ctx->yle_col, yc, ctx->st));
  CTX_TRY(upload(&ctx->yle_val, yv, ctx->st));
  ctx->yle_cap = yv.size();
  if (!ctx->d_w) CTX_TRY(dalloc(&ctx->d_w, 1));
  launch_set_scalar(ctx->d_w, w, ctx->st);
  // LU: b' = b[iperm_r]; x = z[perm_c]
  std::vector<int32_t> gin(n), gout(n);
  for (int64_t i = 0; i < n; ++i) {
    if (perm_r[i] < 0 || perm_r[i] >= n || perm_c[i] < 0 || perm_c[i] >= n)
      return bad(ctx, PEEC_ERR_BADARG, "LU permutation out of range");
    gin[perm_r[i]] = (int32_t)i;
    gout[i] = (int32_t)perm_c[i];
  }
  CTX_TRY(upload(&ctx->g_in, gin, ctx->st));
  CTX_TRY(upload(&ctx->g_out, gout, ctx->st));
  // new factors: a refactorisation plan of the old ones no longer applies
  free_refactor(ctx->rf);
  ctx->have_rf = false;
  ctx->h_gin = gin;
  ctx->h_gout = gout;
  if (row_scale) {
    std::vector<double> rs(row_scale, row_scale + n);
    CTX_TRY(upload(&ctx->lu_rs, rs, ctx->st));
  } else if (ctx->lu_rs) {
    cudaFree(ctx->lu_rs);
    ctx->lu_rs = nullptr;
  }
  CTX_TRY(make_tri(ctx, ctx->Lf, n, L_ptr, L_col, L_val, true));
  CTX_TRY(make_tri(ctx, ctx->Uf, n, U_ptr, U_col, U_val, false));
  CTX_TRY(build_solve_plan(ctx, n));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->have_freq = true;
  return PEEC_OK;
}

// ------------------------------------------------------------------------------------
// device refactorisation (refactor.cu)
// ------------------------------------------------------------------------------------

// position of column c in the sorted columns [b, e) of a CSR row, or -1
static int64_t find_col(const std::vector<int32_t>& col, int64_t b, int64_t e, int32_t c) {
  const auto it = std::lower_bound(col.begin() + b, col.begin() + e, c);
  return (it != col.begin() + e && *it == c) ? it - col.begin() : -1;
}

// Device factorisation of SS from the permutations of the installed host factors (the
// fill-reducing order and the pivot order): the symbolic fill of B = Pr SS Pc without
// further pivoting (up-looking: row p's pattern is B(p,:) joined with U(k,:) for every k
// of L(p,:), in increasing k, new entries left of p joining the queue), installed as
// the solve's factor pattern (levels and solve plan rebuilt); then per slot its SS
// contributions, and per L entry (p, k) the slots of row p that U(k,:) updates; then the
// factors computed on the device at the installed frequency.
static int refactor_run(peec_ctx* ctx);

static int peec_lu_refactor_setup_body(peec_ctx* ctx, int64_t yle_nnz, const int64_t* yle_row,
                                       const int64_t* yle_col) {
  NvtxRange nvtx_range_("peec_lu_refactor_setup");
  if (!ctx || (yle_nnz > 0 && (!yle_row || !yle_col))) return badarg("peec_lu_refactor_setup");
  if (!ctx->have_freq) return bad(ctx, PEEC_ERR_STATE, "no factors installed (peec_set_frequency)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  drop_graphs(ctx);  // the factors and the solve plan are rebuilt below
  free_refactor(ctx->rf);
  ctx->have_rf = false;
  const int64_t n = ctx->n, m = ctx->m, ns = ctx->ns;
  // Yle pattern (CSR, duplicates merged, as set_frequency builds it)
  std::vector<double> zeros(2 * std::max<int64_t>(yle_nnz, 1), 0.0);
  std::vector<int32_t> yp, yc;
  std::vector<c64> yv;
  CTX_TRY(yle_csr(ctx, n, yle_nnz, yle_row, yle_col, zeros.data(), yp, yc, yv));
  // topology on the host
  std::vector<int32_t> e1(m), e2(m), sn(ns);
  cudaMemcpy(e1.data(), ctx->n1, sizeof(int32_t) * m, cudaMemcpyDeviceToHost);
  cudaMemcpy(e2.data(), ctx->n2, sizeof(int32_t) * m, cudaMemcpyDeviceToHost);
  PEEC_CUDA_TRY(cudaMemcpy(sn.data(), ctx->snode, sizeof(int32_t) * ns, cudaMemcpyDeviceToHost));
  std::vector<int32_t> prow(n);  // original row v -> permuted row
  for (int64_t p = 0; p < n; ++p) prow[ctx->h_gin[p]] = (int32_t)p;
  const std::vector<int32_t>& pcol = ctx->h_gout;  // original column u -> permuted column
  // pattern of B, rows of permuted indices
  std::vector<std::vector<int32_t>> brow(n);
  auto add = [&](int32_t v, int32_t u) { brow[prow[v]].push_back(pcol[u]); };
  for (int64_t e = 0; e < m; ++e) {
    add(e1[e], e1[e]); add(e2[e], e2[e]); add(e1[e], e2[e]); add(e2[e], e1[e]);
  }
  for (int64_t i = 0; i < ns; ++i) add(sn[i], sn[i]);
  for (int64_t r = 0; r < n; ++r)
    for (int32_t q = yp[r]; q < yp[r + 1]; ++q) add((int32_t)r, yc[q]);
  // symbolic up-looking factorisation
  std::vector<int64_t> Lp(n + 1, 0), Up(n + 1, 0);
  std::vector<int32_t> Lc, Uc;  // off-diagonal columns, sorted per row
  std::vector<int32_t> mark(n, -1), row;
  for (int64_t p = 0; p < n; ++p) {
    row.clear();
    std::priority_queue<int32_t, std::vector<int32_t>, std::greater<int32_t>> left;
    mark[p] = (int32_t)p;  // the diagonal
    for (int32_t j : brow[p])
      if (mark[j] != p) {
        mark[j] = (int32_t)p;
        row.push_back(j);
        if (j < p) left.push(j);
      }
    while (!left.empty()) {
      const int32_t k = left.top();
      left.pop();
      for (int64_t t = Up[k]; t < Up[k + 1]; ++t) {
        const int32_t j = Uc[t];
        if (mark[j] != p) {
          mark[j] = (int32_t)p;
          row.push_back(j);
          if (j < p) left.push(j);
        }
      }
    }
    std::sort(row.begin(), row.end());
    for (int32_t j : row) (j < p ? Lc : Uc).push_back(j);
    Lp[p + 1] = (int64_t)Lc.size();
    Up[p + 1] = (int64_t)Uc.size();
    if (Lc.size() >= (1u << 30) || Uc.size() >= (1u << 30))
      return bad(ctx, PEEC_ERR_UNSUPPORTED, "factors too large for the device factorisation");
  }
  // install the pattern (diagonal included, placeholder values) with its levels and plan
  {
    auto tri = [&](const std::vector<int64_t>& op, const std::vector<int32_t>& oc, bool lower,
                   LevelTri& T) {
      std::vector<int64_t> ptr(n + 1, 0), col;
      std::vector<double> val;
      col.reserve(oc.size() + n);
      val.reserve(2 * (oc.size() + n));
      for (int64_t r = 0; r < n; ++r) {
        if (!lower) { col.push_back(r); val.push_back(1.0); val.push_back(0.0); }
        for (int64_t t = op[r]; t < op[r + 1]; ++t) {
          col.push_back(oc[t]);
          val.push_back(0.0);
          val.push_back(0.0);
        }
        if (lower) { col.push_back(r); val.push_back(1.0); val.push_back(0.0); }
        ptr[r + 1] = (int64_t)col.size();
      }
      return make_tri(ctx, T, n, ptr.data(), col.data(), val.data(), lower);
    };
    CTX_TRY(tri(Lp, Lc, true, ctx->Lf));
    CTX_TRY(tri(Up, Uc, false, ctx->Uf));
    CTX_TRY(build_solve_plan(ctx, n));
  }
  const LevelTri &L = ctx->Lf, &U = ctx->Uf;
  const int64_t nL = L.hptr[n], nU = U.hptr[n];
  // slot of B entry (p, q): L off-diagonal, diagonal, U off-diagonal
  auto slot = [&](int32_t v, int32_t u) -> int64_t {
    const int32_t p = prow[v], q = pcol[u];
    if (q == p) return nL + p;
    const int64_t at = q < p ? find_col(L.hcol, L.hptr[p], L.hptr[p + 1], q)
                             : find_col(U.hcol, U.hptr[p], U.hptr[p + 1], q);
    if (at < 0) return -1;
    return q < p ? at : nL + n + at;
  };
  const int64_t nslot = nL + n + nU;
  std::vector<std::pair<int64_t, uint32_t>> contrib;
  contrib.reserve(4 * m + ns + yc.size());
  for (int64_t e = 0; e < m; ++e) {
    const int32_t a = e1[e], b = e2[e];
    const int64_t s4[4] = {slot(a, a), slot(b, b), slot(a, b), slot(b, a)};
    for (int t = 0; t < 4; ++t) {
      if (s4[t] < 0) return bad(ctx, PEEC_ERR_STATE, "factor pattern misses an entry of SS");
      contrib.push_back({s4[t], ((t < 2 ? 0u : 1u) << 30) | (uint32_t)e});
    }
  }
  for (int64_t i = 0; i < ns; ++i) {
    const int64_t sl = slot(sn[i], sn[i]);
    if (sl < 0) return bad(ctx, PEEC_ERR_STATE, "factor pattern misses an entry of SS");
    contrib.push_back({sl, (2u << 30) | (uint32_t)i});
  }
  for (int64_t r = 0; r < n; ++r)
    for (int32_t q = yp[r]; q < yp[r + 1]; ++q) {
      const int64_t sl = slot((int32_t)r, yc[q]);
      if (sl < 0) return bad(ctx, PEEC_ERR_STATE, "factor pattern misses an entry of Yle");
      contrib.push_back({sl, (3u << 30) | (uint32_t)q});
    }
  std::stable_sort(contrib.begin(), contrib.end(),
                   [](const std::pair<int64_t, uint32_t>& x, const std::pair<int64_t, uint32_t>& y) {
                     return x.first < y.first;
                   });
  std::vector<int64_t> aptr(nslot + 1, 0);
  std::vector<uint32_t> asrc(contrib.size());
  for (size_t i = 0; i < contrib.size(); ++i) {
    aptr[contrib[i].first + 1]++;
    asrc[i] = contrib[i].second;
  }
  for (int64_t s = 0; s < nslot; ++s) aptr[s + 1] += aptr[s];
  // update targets: for L entry (p, k), each entry (k, j) of U(k,:) lands in row p at j
  std::vector<int32_t> uoff(nL + 1, 0), utgt;
  for (int64_t p = 0; p < n; ++p)
    for (int32_t q = L.hptr[p]; q < L.hptr[p + 1]; ++q) {
      const int32_t k = L.hcol[q];
      for (int32_t t = U.hptr[k]; t < U.hptr[k + 1]; ++t) {
        const int32_t j = U.hcol[t];
        int64_t tg;
        if (j == p) {
          tg = -1;
        } else if (j < p) {
          tg = find_col(L.hcol, L.hptr[p], L.hptr[p + 1], j);
        } else {
          tg = find_col(U.hcol, U.hptr[p], U.hptr[p + 1], j);
          if (tg >= 0) tg |= 0x40000000;
        }
        if (tg < -1 || (tg == -1 && j != p))
          return bad(ctx, PEEC_ERR_STATE, "factor pattern misses a fill entry");
        utgt.push_back((int32_t)tg);
      }
      if (utgt.size() > (size_t)INT32_MAX - 1)
        return bad(ctx, PEEC_ERR_UNSUPPORTED, "device factorisation schedule too long");
      uoff[q + 1] = (int32_t)utgt.size();
    }
  RefactorPlan& R = ctx->rf;
  R.n = n;
  R.nL = nL;
  R.nU = nU;
  R.lvl_off = L.lvl_off;
  std::vector<int32_t> lrows(L.rows.begin(), L.rows.end());
  CTX_TRY(upload(&R.asm_ptr, aptr, ctx->st));
  CTX_TRY(upload(&R.asm_src, asrc, ctx->st));
  CTX_TRY(upload(&R.rows, lrows, ctx->st));
  CTX_TRY(upload(&R.upd_off, uoff, ctx->st));
  if (utgt.empty()) utgt.push_back(0);
  CTX_TRY(upload(&R.upd_tgt, utgt, ctx->st));
  CTX_TRY(dalloc(&R.D, (size_t)n));
  if (!ctx->rf_err) CTX_TRY(dalloc(&ctx->rf_err, 1));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->rf_yp = yp;
  ctx->rf_yc = yc;
  ctx->have_rf = true;
  // the factors at the installed frequency, on the device
  return refactor_run(ctx);
}

// assembles and factorises SS on the device from the state on the device (w, DZ, Yle)
static int refactor_run(peec_ctx* ctx) {
  ctx->have_freq = false;
  PEEC_CUDA_TRY(cudaMemsetAsync(ctx->rf_err, 0, sizeof(int), ctx->st));
  const LevelTri &L = ctx->Lf, &U = ctx->Uf;
  const int nl = refactor_launch(ctx->rf, SfTri{L.ptr, L.col, L.val, L.dinv, L.flag},
                                 SfTri{U.ptr, U.col, U.val, U.dinv, U.flag}, L.val, U.val, ctx->DZ,
                                 ctx->invP, ctx->yle_val, ctx->w, ctx->rf_err, ctx->st);
  if (nl < 0) return nl;
  ctx->launches += nl;
  int herr = 0;
  cudaMemcpyAsync(&herr, ctx->rf_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  if (herr)
    return bad(ctx, PEEC_ERR_UNSUPPORTED,
               "device factorisation met a zero or non-finite pivot: factorise this frequency "
               "on the host (peec_set_frequency)");
  ctx->have_freq = true;
  return PEEC_OK;
}

// Per-frequency state with SS factorised on the device: DZ and Yle as for
// peec_set_frequency (Yle with the pattern given to the set-up), then SS assembled and
// factorised in the plan's pattern and permutations.
static int peec_set_frequency_refactor_body(peec_ctx* ctx, double w, const double* DZ,
                                            int64_t yle_nnz, const int64_t* yle_row,
                                            const int64_t* yle_col, const double* yle_val) {
  NvtxRange nvtx_range_("peec_set_frequency_refactor");
  if (!ctx || !DZ || (yle_nnz > 0 && (!yle_row || !yle_col || !yle_val)))
    return badarg("peec_set_frequency_refactor");
  if (!ctx->have_rf) return bad(ctx, PEEC_ERR_STATE, "no refactorisation plan (peec_lu_refactor_setup)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t n = ctx->n, m = ctx->m;
  std::vector<int32_t> yp, yc;
  std::vector<c64> yv;
  CTX_TRY(yle_csr(ctx, n, yle_nnz, yle_row, yle_col, yle_val, yp, yc, yv));
  if (yp != ctx->rf_yp || yc != ctx->rf_yc)
    return bad(ctx, PEEC_ERR_BADARG, "Yle pattern differs from the one of the refactorisation set-up");
  ctx->have_freq = false;
  ctx->w = w;
  std::vector<c64> dz(m);
  for (int64_t e = 0; e < m; ++e) dz[e] = mk<double>(DZ[2 * e], DZ[2 * e + 1]);
  // The new values go into the arrays in place, and w into its device word, behind the
  // stream's earlier work: every pointer the captured graphs of this context hold stays
  // valid, so they are kept (the factors' pattern, permutations and solve plan do not
  // change either).
  if (!ctx->DZ || !ctx->d_w || ctx->yle_cap != yv.size()) {
    drop_graphs(ctx);
    CTX_TRY(upload(&ctx->DZ, dz, ctx->st));
    CTX_TRY(upload(&ctx->yle_val, yv, ctx->st));
    ctx->yle_cap = yv.size();
    if (!ctx->d_w) CTX_TRY(dalloc(&ctx->d_w, 1));
  } else {
    PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->DZ, dz.data(), sizeof(c64) * m, cudaMemcpyHostToDevice,
                                  ctx->st));
    if (!yv.empty())
      PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->yle_val, yv.data(), sizeof(c64) * yv.size(),
                                    cudaMemcpyHostToDevice, ctx->st));
  }
  launch_set_scalar(ctx->d_w, w, ctx->st);
  return refactor_run(ctx);
}

// Per-edge data from which the device forms DZ at every frequency
// (FFT_solver_QS_S_type.jl:105-114): R and Cd of the four edge halves (m x 4, row-major,
// compute_Z_self.jl), the Lp self terms, the real surface-impedance base Zs0 (the
// frequency's Zs is escal_R * Zs0 * sqrt(w / escal_freq)) and the surface edges.
static int peec_set_edge_state_body(peec_ctx* ctx, const double* R4, const double* Cd4,
                                    const double* Lp_self, const double* Zs0,
                                    const int64_t* surface_edges, int64_t nse, double escal_R,
                                    double escal_freq) {
  if (!ctx || !R4 || !Cd4 || !Lp_self || !Zs0 || (nse > 0 && !surface_edges))
    return badarg("peec_set_edge_state");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  if (!(escal_freq > 0)) return bad(ctx, PEEC_ERR_BADARG, "escal_freq must be positive");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t m = ctx->m;
  std::vector<uint8_t> surf(std::max<int64_t>(m, 1), 0);
  for (int64_t i = 0; i < nse; ++i) {
    if (surface_edges[i] < 0 || surface_edges[i] >= m)
      return bad(ctx, PEEC_ERR_BADARG, "surface edge out of range");
    surf[surface_edges[i]] = 1;
  }
  ctx->have_es = false;
  CTX_TRY(upload(&ctx->es_R4, std::vector<double>(R4, R4 + 4 * m), ctx->st));
  CTX_TRY(upload(&ctx->es_Cd4, std::vector<double>(Cd4, Cd4 + 4 * m), ctx->st));
  CTX_TRY(upload(&ctx->es_Lpd, std::vector<double>(Lp_self, Lp_self + m), ctx->st));
  CTX_TRY(upload(&ctx->es_Zs0, std::vector<double>(Zs0, Zs0 + m), ctx->st));
  CTX_TRY(upload(&ctx->es_surf, surf, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->es_escal_R = escal_R;
  ctx->es_escal_freq = escal_freq;
  ctx->have_es = true;
  return PEEC_OK;
}

// One frequency's state formed on the device: DZ from the edge data, w, Yle (the pattern
// of the refactorisation set-up), and SS assembled and factorised in the plan's pattern.
// Like peec_set_frequency_refactor, it writes in place and keeps the captured graphs.
static int peec_set_frequency_device_body(peec_ctx* ctx, double w, int64_t yle_nnz,
                                          const int64_t* yle_row, const int64_t* yle_col,
                                          const double* yle_val) {
  NvtxRange nvtx_range_("peec_set_frequency_device");
  if (!ctx || (yle_nnz > 0 && (!yle_row || !yle_col || !yle_val)))
    return badarg("peec_set_frequency_device");
  if (!ctx->have_es) return bad(ctx, PEEC_ERR_STATE, "no edge data (peec_set_edge_state)");
  if (!ctx->have_rf) return bad(ctx, PEEC_ERR_STATE, "no refactorisation plan (peec_lu_refactor_setup)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t n = ctx->n, m = ctx->m;
  std::vector<int32_t> yp, yc;
  std::vector<c64> yv;
  CTX_TRY(yle_csr(ctx, n, yle_nnz, yle_row, yle_col, yle_val, yp, yc, yv));
  if (yp != ctx->rf_yp || yc != ctx->rf_yc)
    return bad(ctx, PEEC_ERR_BADARG, "Yle pattern differs from the one of the refactorisation set-up");
  ctx->have_freq = false;
  ctx->w = w;
  if (!ctx->DZ || !ctx->d_w || ctx->yle_cap != yv.size()) {
    drop_graphs(ctx);
    CTX_TRY(dalloc(&ctx->DZ, (size_t)m));
    CTX_TRY(upload(&ctx->yle_val, yv, ctx->st));
    ctx->yle_cap = yv.size();
    if (!ctx->d_w) CTX_TRY(dalloc(&ctx->d_w, 1));
  } else if (!yv.empty()) {
    PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->yle_val, yv.data(), sizeof(c64) * yv.size(),
                                  cudaMemcpyHostToDevice, ctx->st));
  }
  launch_edge_dz(m, ctx->es_R4, ctx->es_Cd4, ctx->es_Lpd, ctx->es_Zs0, ctx->es_surf,
                 ctx->es_escal_R, std::sqrt(w / ctx->es_escal_freq), w, ctx->DZ, ctx->st);
  launch_set_scalar(ctx->d_w, w, ctx->st);
  ctx->launches += 2;
  return refactor_run(ctx);
}

// ------------------------------------------------------------------------------------
// operator
// ------------------------------------------------------------------------------------

static void lu_solve(peec_ctx* ctx, const c64* b, c64* x) {
  const int n = (int)ctx->n;
  const LevelTri &L = ctx->Lf, &U = ctx->Uf;
  ctx->launches += launch_sptrsv(
      ctx->grp, ctx->st2, ctx->ev_fork, ctx->ev_join, ctx->sf_ord, ctx->sf_nL, ctx->sf_total, SfTri{L.ptr, L.col, L.val, L.dinv, L.flag},
      SfTri{U.ptr, U.col, U.val, U.dinv, U.flag}, b, ctx->g_in, ctx->lu_rs, ctx->lutmp,
      ctx->lutmp2, ctx->sf_ctl, ctx->st);
  launch_perm_gather(ctx->lutmp2, ctx->g_out, nullptr, n, x, ctx->st);
  ctx->launches += 1;
}

// A triangular-solve wait that ran into its limit leaves an error word on the device;
// entry points read it once their work is complete.
static int check_solve_errors(peec_ctx* ctx) {
  int e = 0, ez = 0;
  if (ctx->sf_ctl)
    PEEC_CUDA_TRY(cudaMemcpyAsync(&e, ctx->sf_ctl + 2, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  if (ctx->zerr)
    PEEC_CUDA_TRY(cudaMemcpyAsync(&ez, ctx->zerr, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  if (e) {
    cudaMemsetAsync(ctx->sf_ctl + 2, 0, sizeof(int), ctx->st);
    return bad(ctx, PEEC_ERR_TIMEOUT, "LU solve: a row dependency wait ran into its limit");
  }
  if (ez) {
    cudaMemsetAsync(ctx->zerr, 0, sizeof(int), ctx->st);
    return bad(ctx, PEEC_ERR_TIMEOUT, "z pass: a staged tile copy wait ran into its limit");
  }
  return PEEC_OK;
}

// enqueue the sparse half of an operator application y = M^-1 K x (block rows, the LU
// solve of the preconditioner), given the convolutions LpI = Lp*I and PQ = P*Q of x
static void sparse_enqueue(peec_ctx* ctx, const c64* x, c64* y, const c64* LpI, const c64* PQ) {
  const int64_t m = ctx->m, ns = ctx->ns, n = ctx->n;
  cudaStream_t st = ctx->st;
  const c64* I = x;
  const c64* Q = x + m;
  const c64* Phi = x + m + ns;
  launch_edge_rows(I, Phi, LpI, ctx->DZ, ctx->n1, ctx->n2, ctx->d_w, (int)m, ctx->Y1, ctx->U1, st);
  launch_surf_rows(PQ, Phi, ctx->snode, ctx->invP, (int)ns, ctx->Y2, ctx->U2, st);
  launch_node_rows(I, Q, Phi, ctx->U1, ctx->U2, ctx->ne_ptr, ctx->ne_idx, ctx->nsn_ptr,
                   ctx->nsn_idx, ctx->yle_ptr, ctx->yle_col, ctx->yle_val, ctx->d_w, (int)n,
                   ctx->tvec, st);
  ctx->launches += 3;
  lu_solve(ctx, ctx->tvec, ctx->Mvec);
  launch_final_rows(ctx->Y1, ctx->Y2, ctx->Mvec, ctx->DZ, ctx->n1, ctx->n2, ctx->snode, ctx->invP,
                    (int)m, (int)ns, (int)n, y, st);
  ctx->launches++;
}

// enqueue one operator application y = M^-1 K x on the context stream
static int matvec_enqueue(peec_ctx* ctx, const c64* x, c64* y, int prec, bool events) {
  cudaStream_t st = ctx->st;
  if (events) cudaEventRecord(ctx->ev[0], st);
  if (ctx->dense) {
    // Lp blocks (without their diagonals) and P: FP32 copies for the FP32 operator, FP64
    // for the others (more accurate than float-float, at FP64 speed). The pass events of
    // a profile put the products in the z-pass slot.
    const bool f32 = prec == PEEC_PREC_FP32;
    cudaEvent_t* pe = ctx->prof ? ctx->pev.data() : nullptr;
    if (pe) for (int e = 0; e < 3; ++e) cudaEventRecord(pe[e], st);
    const int64_t off[3] = {0, ctx->mx, ctx->mx + ctx->my};
    const int64_t sz[3] = {ctx->mx, ctx->my, ctx->mz};
    if (ctx->dense_rcc && !ctx->dense_rcc_ready)
      return bad(ctx, PEEC_ERR_STATE, "retarded blocks not formed (peec_set_dense_rcc_frequency)");
    // the three Lp blocks on st2, beside P on st (fork and join events; under capture,
    // graph edges): the small blocks' products and reductions hide behind P's stream
    const bool fork = ctx->st2 && ctx->m > 0;
    cudaStream_t sl = fork ? ctx->st2 : st;
    c64* part_lp = ctx->dn_part;
    c64* part_p = ctx->dn_part + ctx->dn_part_half;
    if (fork) {
      cudaEventRecord(ctx->ev_fork, st);
      cudaStreamWaitEvent(ctx->st2, ctx->ev_fork, 0);
    }
    for (int b = 0; b < 3; ++b) {
      if (ctx->dense_rcc)
        ctx->launches += dense_apply_c(f32 ? (const void*)ctx->dnc32[b] : (const void*)ctx->dnc64[b],
                                       f32, sz[b], ctx->dn_ld[b], x + off[b], 1, part_lp,
                                       ctx->LpI + off[b], sl);
      else
        ctx->launches += dense_apply(f32 ? (const void*)ctx->dn32[b] : (const void*)ctx->dn64[b],
                                     f32, sz[b], ctx->dn_ld[b], x + off[b], 1, part_lp,
                                     ctx->LpI + off[b], sl);
    }
    if (fork) cudaEventRecord(ctx->ev_join, ctx->st2);
    if (ctx->dense_rcc)
      ctx->launches += dense_apply_c(f32 ? (const void*)ctx->dnc32[3] : (const void*)ctx->dnc64[3],
                                     f32, ctx->ns, ctx->dn_ld[3], x + ctx->m, 0, part_p, ctx->PQ,
                                     st);
    else
      ctx->launches += dense_apply(f32 ? (const void*)ctx->dn32[3] : (const void*)ctx->dn64[3], f32,
                                   ctx->ns, ctx->dn_ld[3], x + ctx->m, 0, part_p, ctx->PQ, st);
    if (fork) cudaStreamWaitEvent(st, ctx->ev_join, 0);
    if (pe) for (int e = 3; e < 6; ++e) cudaEventRecord(pe[e], st);
    if (events) cudaEventRecord(ctx->ev[1], st);
    sparse_enqueue(ctx, x, y, ctx->LpI, ctx->PQ);
    if (events) cudaEventRecord(ctx->ev[2], st);
    return PEEC_OK;
  }
  const void* tw[3] = {ctx->tw64, ctx->tw32, ctx->twff};
  const void* ph[6] = {ctx->ph64[0], ctx->ph64[1], ctx->ph64[2],
                       ctx->ph32[0], ctx->ph32[1], ctx->ph32[2]};
  CTX_TRY(conv_all(ctx->fam, 6, ctx->spec, ph, x, ctx->LpI, ctx->PQ, ctx->m, prec, tw,
                   ctx->twmax, st, ctx->prof ? ctx->pev.data() : nullptr, &ctx->zt));
  if (ctx->rcc) {
    // the imaginary-part rows' convolutions, joined as LpI += i LpI2, PQ += i PQ2
    CTX_TRY(conv_all(ctx->fam, 6, ctx->spec_im, ph, x, ctx->LpI2, ctx->PQ2, ctx->m, prec, tw,
                     ctx->twmax, st, nullptr, &ctx->zt));
    launch_add_i(ctx->LpI2, ctx->m, ctx->LpI, st);
    launch_add_i(ctx->PQ2, ctx->ns, ctx->PQ, st);
    ctx->launches += 2;
  }
  // one launch per x / y pass over all families, the shared z pass of the face
  // families, and the edge families' z passes: one launch over all of them in the staged
  // FP32 form (ZTune form 2), else one per family
  int nedge = 0;
  for (const auto& F : ctx->fam) nedge += (F.active && F.lp) ? 1 : 0;
  const bool edge_one = prec == PEEC_PREC_FP32 && ctx->zt.edge == 2 && zpass_yz_edges(ctx->fam, 6);
  ctx->launches += (5 + (edge_one ? (nedge > 0) : nedge)) * (ctx->rcc ? 2 : 1);
  if (events) cudaEventRecord(ctx->ev[1], st);
  sparse_enqueue(ctx, x, y, ctx->LpI, ctx->PQ);
  if (events) cudaEventRecord(ctx->ev[2], st);
  return PEEC_OK;
}

static int matvec_dev(peec_ctx* ctx, const c64* x, c64* y, int prec, bool timed) {
  if (!ctx->have_topo || !ctx->have_spec || !ctx->have_freq || !ctx->have_pdiag)
    return bad(ctx, PEEC_ERR_STATE, "operator incomplete (topology, pdiag, rows, frequency)");
  if (timed || ctx->prof || !ctx->use_graphs) {
    CTX_TRY(matvec_enqueue(ctx, x, y, prec, timed));
  } else {
    auto& ge = ctx->graphs[std::make_tuple((const void*)x, (void*)y, prec)];
    if (ge.exec) {
      PEEC_CUDA_TRY(cudaGraphLaunch(ge.exec, ctx->st));
      ctx->launches += ge.kernels;
    } else if (ge.calls++ == 0) {
      // first application with these buffers runs eagerly (one-time kernel set-up)
      CTX_TRY(matvec_enqueue(ctx, x, y, prec, false));
    } else {
      const int64_t l0 = ctx->launches;
      cudaGraph_t g = nullptr;
      PEEC_CUDA_TRY(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
      const int rc = matvec_enqueue(ctx, x, y, prec, false);
      const cudaError_t ec = cudaStreamEndCapture(ctx->st, &g);
      if (rc != PEEC_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (ec != cudaSuccess) return fail_cuda(ec, "cudaStreamEndCapture", __FILE__, __LINE__);
      const cudaError_t ei = cudaGraphInstantiate(&ge.exec, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) return fail_cuda(ei, "cudaGraphInstantiate", __FILE__, __LINE__);
      ge.kernels = ctx->launches - l0;
      PEEC_CUDA_TRY(cudaGraphLaunch(ge.exec, ctx->st));
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda(e, "matvec launch", __FILE__, __LINE__);
  return PEEC_OK;
}

static int peec_matvec_dev_body(peec_ctx* ctx, const void* x, void* y, int precision) {
  NvtxRange nvtx_range_("peec_matvec_dev");
  if (!ctx || !x || !y) return badarg("peec_matvec_dev");
  if (precision < 0 || precision > 2) return bad(ctx, PEEC_ERR_BADARG, "precision must be 0, 1 or 2");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  CTX_TRY(matvec_dev(ctx, (const c64*)x, (c64*)y, precision, true));
  PEEC_CUDA_TRY(cudaEventSynchronize(ctx->ev[2]));
  cudaEventElapsedTime(&ctx->t_total, ctx->ev[0], ctx->ev[2]);
  cudaEventElapsedTime(&ctx->t_conv, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&ctx->t_sparse, ctx->ev[1], ctx->ev[2]);
  CTX_TRY(check_solve_errors(ctx));
  return PEEC_OK;
}

static int peec_matvec_body(peec_ctx* ctx, const double* x, double* y, int precision) {
  NvtxRange nvtx_range_("peec_matvec");
  if (!ctx || !x || !y) return badarg("peec_matvec");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const size_t bytes = sizeof(c64) * ctx->N;
  PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->dx, x, bytes, cudaMemcpyHostToDevice, ctx->st));
  CTX_TRY(peec_matvec_dev(ctx, ctx->dx, ctx->dy, precision));
  PEEC_CUDA_TRY(cudaMemcpyAsync(y, ctx->dy, bytes, cudaMemcpyDeviceToHost, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return PEEC_OK;
}

extern "C" void* peec_stream(const peec_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }

extern "C" int peec_conv_count(const peec_ctx* ctx) { return ctx ? 6 : 0; }

extern "C" int peec_set_zpass_forms(peec_ctx* ctx, int face, int edge, int edge_plan) {
  if (!ctx) return badarg(__func__);
  if (face < 0 || face > 2 || edge < 0 || edge > 2 || edge_plan < 0 || edge_plan > 1)
    return bad(ctx, PEEC_ERR_BADARG, "z-pass forms are 0..2 and edge plans 0..1");
  drop_graphs(ctx);
  ctx->zt.face = face;
  ctx->zt.edge = edge;
  ctx->zt.edge_plan = edge_plan;
  return PEEC_OK;
}

extern "C" int peec_zpass_tuning(const peec_ctx* ctx, int choice[3], double face_ms[3],
                                 double edge_ms[6]) {
  if (!ctx) return badarg(__func__);
  if (choice) {
    choice[0] = zpass_yz_faces(ctx->fam, 6) ? ctx->zt.face : 0;
    choice[1] = zpass_yz_edges(ctx->fam, 6) ? ctx->zt.edge : 0;
    choice[2] = ctx->zt.edge_plan;
  }
  if (face_ms) std::memcpy(face_ms, ctx->zface_ms, sizeof(ctx->zface_ms));
  if (edge_ms) std::memcpy(edge_ms, ctx->zedge_ms, sizeof(ctx->zedge_ms));
  return PEEC_OK;
}

extern "C" int peec_conv_info(const peec_ctx* ctx, int i, int* L, int* dims, int* active,
                              int* kind) {
  if (!ctx || i < 0 || i >= 6) return badarg(__func__);
  const Family& F = ctx->fam[i];
  for (int k = 0; k < 3; ++k) {
    if (L) L[k] = F.L[k];
    if (dims) dims[k] = F.dims[k];
  }
  if (active) *active = F.active ? 1 : 0;
  if (kind) *kind = F.lp ? 1 : 0;
  return PEEC_OK;
}

static int peec_profile_matvec_body(peec_ctx* ctx, int precision, int iters, double* ms) {
  if (!ctx || !ms || iters < 1) return badarg("peec_profile_matvec");
  if (precision < 0 || precision > 2) return bad(ctx, PEEC_ERR_BADARG, "precision must be 0, 1 or 2");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  if (ctx->pev.size() != 6) {
    for (auto e : ctx->pev) cudaEventDestroy(e);
    ctx->pev.assign(6, nullptr);
    for (auto& e : ctx->pev) PEEC_CUDA_TRY(cudaEventCreate(&e));
  }
  double acc[7] = {0, 0, 0, 0, 0, 0, 0};
  // one untimed application first: kernel modules load lazily at their first launch
  CTX_TRY(matvec_dev(ctx, ctx->dx, ctx->dy, precision, true));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  ctx->prof = true;
  for (int it = 0; it < iters; ++it) {
    int rc = matvec_dev(ctx, ctx->dx, ctx->dy, precision, true);
    if (rc) {
      ctx->prof = false;
      return rc;
    }
    PEEC_CUDA_TRY(cudaEventSynchronize(ctx->ev[2]));
    float t;
    for (int c = 0; c < 5; ++c) {
      cudaEventElapsedTime(&t, ctx->pev[c], ctx->pev[c + 1]);
      acc[c] += t;
    }
    cudaEventElapsedTime(&t, ctx->ev[1], ctx->ev[2]);
    acc[5] += t;
    cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[2]);
    acc[6] += t;
  }
  ctx->prof = false;
  for (int c = 0; c < 7; ++c) ms[c] = acc[c] / iters;
  CTX_TRY(check_solve_errors(ctx));
  return PEEC_OK;
}

static int peec_multidot_body(peec_ctx* ctx, const void* U, int64_t ldu, const void* v, int64_t N,
                             int k, void* out) {
  if (!ctx || !U || !v || !out || N < 1 || k < 1 || ldu < N)
    return PEEC_ERR_BADARG;
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const size_t need = (size_t)red_blocks((size_t)N) * (size_t)k;
  if (ctx->mdcap < need) {
    if (ctx->mdpart) cudaFree(ctx->mdpart);
    ctx->mdpart = nullptr;
    PEEC_CUDA_TRY(cudaMalloc(&ctx->mdpart, need * sizeof(c64)));
    ctx->mdcap = need;
  }
  ctx->launches += launch_multidot((const c64*)U, (size_t)ldu, (const c64*)v, (size_t)N, k,
                                   ctx->mdpart, (c64*)out, ctx->st);
  PEEC_CUDA_TRY(cudaGetLastError());
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return PEEC_OK;
}

extern "C" int peec_last_timing(peec_ctx* ctx, double* total_ms, double* conv_ms,
                                double* sparse_ms) {
  if (!ctx) return badarg(__func__);
  if (total_ms) *total_ms = ctx->t_total;
  if (conv_ms) *conv_ms = ctx->t_conv;
  if (sparse_ms) *sparse_ms = ctx->t_sparse;
  return PEEC_OK;
}

static int peec_port_rhs_body(peec_ctx* ctx, int64_t n1, int64_t n2, double Is, double* tn) {
  NvtxRange nvtx_range_("peec_port_rhs");
  if (!ctx || !tn) return badarg("peec_port_rhs");
  if (!ctx->have_freq || !ctx->have_pdiag) return bad(ctx, PEEC_ERR_STATE, "frequency state not set");
  if (n1 < 0 || n1 >= ctx->n || n2 < 0 || n2 >= ctx->n) return bad(ctx, PEEC_ERR_BADARG, "port node out of range");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t m = ctx->m, ns = ctx->ns, n = ctx->n;
  std::vector<c64> is(n, mk<double>(0, 0));
  is[n1] = mk<double>(Is, 0);
  is[n2] = mk<double>(-Is, 0);
  PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->tvec, is.data(), sizeof(c64) * n, cudaMemcpyHostToDevice, ctx->st));
  lu_solve(ctx, ctx->tvec, ctx->Mvec);
  // Y1 = Y2 = 0 gives y1 = -invZ*A*M, y2 = invP*Gamma'*M, y3 = M
  PEEC_CUDA_TRY(cudaMemsetAsync(ctx->Y1, 0, sizeof(c64) * (m > 0 ? m : 1), ctx->st));
  PEEC_CUDA_TRY(cudaMemsetAsync(ctx->Y2, 0, sizeof(c64) * (ns > 0 ? ns : 1), ctx->st));
  launch_final_rows(ctx->Y1, ctx->Y2, ctx->Mvec, ctx->DZ, ctx->n1, ctx->n2, ctx->snode, ctx->invP,
                    (int)m, (int)ns, (int)n, ctx->dy, ctx->st);
  ctx->launches++;
  PEEC_CUDA_TRY(cudaMemcpyAsync(tn, ctx->dy, sizeof(c64) * ctx->N, cudaMemcpyDeviceToHost, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  return PEEC_OK;
}

static int peec_check_wait_limit_body(peec_ctx* ctx) {
  if (!ctx) return badarg("peec_check_wait_limit");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  int e = 0;
  const int rc = selftest_wait_limit(1 << 16, ctx->st, &e);
  if (rc) return ctx->err = g_err, rc;
  ctx->launches += 2;
  if (e) return bad(ctx, PEEC_ERR_TIMEOUT, "self-test: a dependency wait ran into its limit");
  return PEEC_OK;
}

static int peec_adjoint_body(peec_ctx* ctx, const double* x, const int32_t* v1,
                            const int32_t* v2, const double* d1, const double* d2, double Is,
                            int64_t nvox, double* g) {
  NvtxRange nvtx_range_("peec_adjoint");
  if (!ctx || !x || !v1 || !v2 || !d1 || !d2 || !g || nvox < 0 || Is == 0)
    return badarg("peec_adjoint");
  if (!ctx->have_topo) return bad(ctx, PEEC_ERR_STATE, "topology not set");
  if (!ctx->lattice) return bad(ctx, PEEC_ERR_STATE, "no voxel lattice (peec_set_incidence topology)");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const int64_t m = ctx->m;
  int32_t *dv1 = nullptr, *dv2 = nullptr;
  c64 *dd1 = nullptr, *dd2 = nullptr;
  double* dg = nullptr;
  int rc = PEEC_OK;
  auto cleanup = [&]() {
    cudaFree(dv1);
    cudaFree(dv2);
    cudaFree(dd1);
    cudaFree(dd2);
    cudaFree(dg);
  };
  if (dalloc(&dv1, m) || dalloc(&dv2, m) || dalloc(&dd1, m) || dalloc(&dd2, m) ||
      dalloc(&dg, 2 * (size_t)std::max<int64_t>(nvox, 1))) {
    cleanup();
    return bad(ctx, PEEC_ERR_OOM, "peec_adjoint: device buffers");
  }
  cudaStream_t st = ctx->st;
  cudaMemcpyAsync(ctx->dx, x, sizeof(c64) * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dv1, v1, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dv2, v2, sizeof(int32_t) * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dd1, d1, sizeof(c64) * m, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dd2, d2, sizeof(c64) * m, cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(dg, 0, sizeof(double) * 2 * (size_t)std::max<int64_t>(nvox, 1), st);
  launch_adjoint(ctx->dx, dv1, dv2, dd1, dd2, 2.0 / Is, m, nvox, dg, st);
  ctx->launches++;
  cudaError_t e = cudaGetLastError();  // launch configuration errors are not sticky
  if (e == cudaSuccess) {
    cudaMemcpyAsync(g, dg, sizeof(double) * 2 * (size_t)nvox, cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
  } else {
    cudaStreamSynchronize(st);  // the uploads above still read caller memory
  }
  if (e != cudaSuccess) rc = fail_cuda(e, "peec_adjoint", __FILE__, __LINE__);
  cleanup();
  return rc;
}

// ------------------------------------------------------------------------------------
// Householder GMRES (gmres_custom.jl:1-331) on device vectors
// ------------------------------------------------------------------------------------

// work vectors for Krylov solves of up to k reflectors, and the reflector basis in the
// storage the solve's precision uses (complex float-float for the FP32-operator solves)
static int ensure_krylov(peec_ctx* ctx, int k, int prec) {
  const size_t N = ctx->N;
  if (prec == PEEC_PREC_FP32) {
    if (ctx->kcap_u32 < k) {
      drop_krylov_graphs(ctx);
      CTX_TRY(dalloc(&ctx->U32, N * (size_t)k));
      ctx->kcap_u32 = k;
    }
  } else if (ctx->kcap_u < k) {
    drop_krylov_graphs(ctx);
    CTX_TRY(dalloc(&ctx->U, N * (size_t)k));
    ctx->kcap_u = k;
  }
  if (ctx->kcap >= k) return PEEC_OK;
  drop_krylov_graphs(ctx);
  for (c64** p : {&ctx->gb, &ctx->gx, &ctx->gr, &ctx->gv, &ctx->gw, &ctx->gxm, &ctx->gxmin,
                  &ctx->gtmp, &ctx->gzero})
    CTX_TRY(dalloc(p, N));
  PEEC_CUDA_TRY(cudaMemsetAsync(ctx->gzero, 0, sizeof(c64) * N, ctx->st));
  CTX_TRY(dalloc(&ctx->dcoef, 2 * (size_t)k + 16));  // xupdate stages 2k coefficients
  CTX_TRY(dalloc(&ctx->dcoef2, 2 * (size_t)k + 16));
  CTX_TRY(dalloc(&ctx->dT, (size_t)k * k));            // compact-WY T, ld = k
  const int nb = red_blocks(N);
  CTX_TRY(dalloc(&ctx->dpart, (size_t)nb * (k + 8)));
  CTX_TRY(dalloc(&ctx->dred, nb + 8));
  CTX_TRY(dalloc(&ctx->dscal, 16));
  ctx->kcap = k;
  return PEEC_OK;
}

// byte offsets of the arrays of a cycle state with `inner` iterations (16-byte aligned)
struct GmLayout {
  size_t res, wv, J, Utop, R, total;
};
static GmLayout gm_layout(int inner) {
  auto up16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
  GmLayout L;
  size_t o = up16(sizeof(GmDev));
  L.res = o;
  o = up16(o + sizeof(double) * ((size_t)inner + 2));
  L.wv = o;
  o += sizeof(c64) * ((size_t)inner + 1);
  L.J = o;
  o += sizeof(c64) * 2 * (size_t)inner;
  L.Utop = o;
  o += sizeof(c64) * ((size_t)inner + 1) * ((size_t)inner + 1);
  L.R = o;
  o += sizeof(c64) * (size_t)inner * inner;
  L.total = o;
  return L;
}

static int ensure_gm(peec_ctx* ctx, int inner) {
  if (ctx->gm_inner == inner && ctx->gm_block) return PEEC_OK;
  drop_krylov_graphs(ctx);
  const GmLayout L = gm_layout(inner);
  CTX_TRY(dalloc(&ctx->gm_block, L.total));
  if (ctx->gm_up) cudaFreeHost(ctx->gm_up);
  if (ctx->gm_down) cudaFreeHost(ctx->gm_down);
  ctx->gm_up = ctx->gm_down = nullptr;
  ctx->gm_inner = -1;
  PEEC_CUDA_TRY(cudaMallocHost(&ctx->gm_up, sizeof(GmDev)));
  PEEC_CUDA_TRY(cudaMallocHost(&ctx->gm_down, L.J));
  ctx->gm_inner = inner;
  return PEEC_OK;
}

// whether the operator application (x, y, prec) has run once outside a capture, so that
// its one-time set-up is done and it may be captured
static bool matvec_warm(peec_ctx* ctx, const c64* x, c64* y, int prec) {
  auto it = ctx->graphs.find(std::make_tuple((const void*)x, (void*)y, prec));
  return it != ctx->graphs.end() && (it->second.calls > 0 || it->second.exec);
}

// The graph of the device loop: a WHILE conditional node whose body is one Arnoldi
// iteration (v = P1..Pj e_j, w = A v, orthogonalisation, scalar step, new reflector).
// The condition starts at 1 on every launch, so the body runs at least once; the scalar
// step sets it after every iteration.
static int build_krylov_graph(peec_ctx* ctx, GmBody B, int prec, int inner) {
  peec_ctx::KrylovGraph& kg = ctx->kg[prec];
  if (kg.exec) cudaGraphExecDestroy(kg.exec);
  kg = peec_ctx::KrylovGraph();
  cudaGraph_t g = nullptr;
  PEEC_CUDA_TRY(cudaGraphCreate(&g, 0));
  auto fail = [&](cudaError_t e, const char* what) {
    cudaGraphDestroy(g);
    return fail_cuda(e, what, __FILE__, __LINE__);
  };
  cudaGraphConditionalHandle h = 0;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return fail(e, "cudaGraphConditionalHandleCreate");
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (e != cudaSuccess) return fail(e, "cudaGraphAddNode (while)");
  cudaGraph_t body = np.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(ctx->st, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "cudaStreamBeginCaptureToGraph");
  B.cond = h;
  B.use_cond = 1;
  const int64_t l0 = ctx->launches;
  ctx->launches += gm_pre(B);
  const int rc = matvec_enqueue(ctx, B.v, B.w, prec, false);
  ctx->launches += gm_post(B);
  const int64_t kernels = ctx->launches - l0;
  ctx->launches = l0;
  cudaGraph_t cap = nullptr;
  e = cudaStreamEndCapture(ctx->st, &cap);
  if (rc != PEEC_OK) {
    cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(e, "cudaStreamEndCapture (while body)");
  e = cudaGraphInstantiate(&kg.exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    kg.exec = nullptr;
    return fail_cuda(e, "cudaGraphInstantiate (device loop)", __FILE__, __LINE__);
  }
  kg.inner = inner;
  kg.kernels = kernels;
  return PEEC_OK;
}

// Runs Arnoldi iterations of the current cycle from the state's iteration index: as one
// launch of the device-loop graph (iterations until the scalar step ends the loop), or
// one iteration of eager launches (the first application of the operator on these
// buffers, profiling, or the device loop switched off). *graph_kernels: kernels per
// iteration of a graph launch, 0 for an eager iteration (counted here).
static int gm_iterate(peec_ctx* ctx, GmBody& B, int prec, int inner, int64_t* graph_kernels) {
  *graph_kernels = 0;
  if (ctx->dev_loop && !ctx->prof && matvec_warm(ctx, B.v, B.w, prec)) {
    peec_ctx::KrylovGraph& kg = ctx->kg[prec];
    if (!kg.exec || kg.inner != inner) CTX_TRY(build_krylov_graph(ctx, B, prec, inner));
    PEEC_CUDA_TRY(cudaGraphLaunch(kg.exec, ctx->st));
    *graph_kernels = kg.kernels;
    ctx->kg_launches++;
    return PEEC_OK;
  }
  B.use_cond = 0;
  ctx->launches += gm_pre(B);
  CTX_TRY(matvec_dev(ctx, B.v, B.w, prec, false));
  ctx->launches += gm_post(B);
  PEEC_CUDA_TRY(cudaGetLastError());
  return PEEC_OK;
}

namespace {

// Host side of the Householder GMRES. Vectors of length N live on the device; the
// compact-WY matrix T (reflector products P1..Pk = I - U T U^H) lives on the device
// and is only touched by small kernels; so does the scalar work of an iteration
// (k_gm_step: reflector heads, Givens rotations, R, w, the residual estimate). The host
// runs the reference's control flow around it: the convergence checks on the true
// residual, stagnation, restarts. Host -> device coefficient vectors go through a ring
// of pinned slots.
struct Gm {
  peec_ctx* ctx;
  size_t N;
  int prec;
  cudaStream_t st;
  int rc = PEEC_OK;
  int ring = 0;
  int pending = 0;  // uploads queued since the last stream synchronisation

  void sync() {
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == PEEC_OK)
      rc = fail_cuda(cudaGetLastError(), "sync", __FILE__, __LINE__);
    pending = 0;
  }

  double norm(const c64* v, size_t i0 = 0) {
    launch_norm2(v, N, i0, ctx->dred, ctx->dscal, st);
    ctx->launches += 2;
    cudaMemcpyAsync(ctx->hscal, ctx->dscal, sizeof(double), cudaMemcpyDeviceToHost, st);
    sync();
    return std::sqrt(ctx->hscal[0]);
  }
  void matvec(const c64* x, c64* y) {
    if (rc == PEEC_OK) rc = matvec_dev(ctx, x, y, prec, false);
  }
  void residual(const c64* b, const c64* x, c64* out) {  // out = b - A x
    matvec(x, ctx->gtmp);
    launch_sub(b, ctx->gtmp, N, out, st);
    ctx->launches++;
  }
  void copy(c64* dst, const c64* src) {
    cudaMemcpyAsync(dst, src, sizeof(c64) * N, cudaMemcpyDeviceToDevice, st);
  }
  // asynchronous upload through the pinned ring (slots of kSlot entries)
  void to_dev(c64* d, const std::vector<cd>& h) {
    if (pending == kSlots) sync();  // every slot may still feed a queued copy
    pending++;
    const size_t slot = (size_t)(ring++ % kSlots) * kSlot;
    for (size_t i = 0; i < h.size(); ++i)
      ctx->hsmall[slot + i] = mk<double>(h[i].real(), h[i].imag());
    cudaMemcpyAsync(d, ctx->hsmall + slot, sizeof(c64) * h.size(), cudaMemcpyHostToDevice, st);
  }
  std::vector<cd> from_dev(const c64* d, size_t cnt) {
    cudaMemcpyAsync(ctx->hread, d, sizeof(c64) * cnt, cudaMemcpyDeviceToHost, st);
    sync();
    std::vector<cd> h(cnt);
    for (size_t i = 0; i < cnt; ++i) h[i] = cd(ctx->hread[i].x, ctx->hread[i].y);
    return h;
  }
  static constexpr int kSlots = 16;
  static constexpr int kSlot = 4096;
};

cd sgn(cd d) {
  if (d == cd(0.0, 0.0)) return cd(1.0, 0.0);
  return d / std::abs(d);
}

// solve upper-triangular R(0:k,0:k) y = rhs (R column-major with leading dim ld)
std::vector<cd> utri_solve(const std::vector<cd>& R, int ld, int k, std::vector<cd> rhs) {
  for (int i = k - 1; i >= 0; --i) {
    cd s = rhs[i];
    for (int j = i + 1; j < k; ++j) s -= R[(size_t)j * ld + i] * rhs[j];
    rhs[i] = s / R[(size_t)i * ld + i];
  }
  return rhs;
}

}  // namespace

// out = base + Q_k [y; 0] = base + [y;0] - U(:,0:k) (T_k (Utop(0:k,0:k)^H y))
static void apply_Q(Gm& g, const std::vector<cd>& Utop, int ldt, int k, const std::vector<cd>& y,
                    const c64* base, c64* out) {
  peec_ctx* ctx = g.ctx;
  std::vector<cd> h(k);
  for (int col = 0; col < k; ++col) {
    cd s = 0;
    for (int row = 0; row < k; ++row) s += std::conj(Utop[(size_t)col * ldt + row]) * y[row];
    h[col] = s;
  }
  std::vector<cd> yy(y.begin(), y.begin() + k);
  g.to_dev(ctx->dcoef2, h);
  g.to_dev(ctx->dcoef + k, yy);
  launch_tri(ctx->dT, ctx->kcap, k, ctx->dcoef2, ctx->dcoef, 0, g.st);  // c = T h
  if (g.prec == PEEC_PREC_FP32)
    launch_xupdate(base ? base : ctx->gzero, ctx->U32, g.N, ctx->dcoef, ctx->dcoef + k, k, g.N,
                   out, g.st);
  else
    launch_xupdate(base ? base : ctx->gzero, ctx->U, g.N, ctx->dcoef, ctx->dcoef + k, k, g.N, out,
                   g.st);
  ctx->launches += 2;
}

// x0_zero: the caller guarantees x_dev == 0, so the initial residual is b itself (A*0 is
// exactly 0 in every precision) and its operator application is skipped. Convergence is
// always confirmed on the true residual, as gmres_custom does: deciding on the recursive
// estimate alone left port impedances of the mixed solve a little less accurate at
// ill-conditioned frequencies.
static int gmres_run(peec_ctx* ctx, const c64* b_dev, c64* x_dev, double tol, int maxit,
                     int restarted, int restart, int prec, int* flag_out, double* relres_out,
                     int* iter_out, std::vector<double>& resvec_out, bool x0_zero = false) {
  const size_t N = ctx->N;
  int n = (int)N;
  int outer, inner;
  if (restarted) {
    outer = maxit;
    inner = std::min(restart, n);
  } else {
    outer = 1;
    if (maxit > n) maxit = n;
    inner = maxit;
  }
  if (inner < 1) inner = 1;
  if (2 * (inner + 1) > Gm::kSlot) return bad(ctx, PEEC_ERR_UNSUPPORTED, "inner iterations above 2047");
  CTX_TRY(ensure_krylov(ctx, inner + 1, prec));
  Gm g{ctx, N, prec, ctx->st};
  const int ldT = ctx->kcap;
  // FP32-operator solves keep their reflectors in complex float-float, with float-float
  // arithmetic in the basis kernels; FP64 and float-float-operator solves in complex double
  const bool f32 = prec == PEEC_PREC_FP32;
  c64 *b = ctx->gb, *x = ctx->gx, *r = ctx->gr, *v = ctx->gv, *xm = ctx->gxm,
      *xmin = ctx->gxmin, *add = ctx->gw;
  g.copy(b, b_dev);
  g.copy(x, x_dev);
  const double n2b = g.norm(b);
  if (g.rc) return g.rc;
  if (n2b == 0) {
    cudaMemsetAsync(x_dev, 0, sizeof(c64) * N, ctx->st);
    cudaStreamSynchronize(ctx->st);
    *flag_out = 0; *relres_out = 0; iter_out[0] = iter_out[1] = 0;
    resvec_out.assign(1, 0.0);
    return PEEC_OK;
  }
  int flag = 1;
  g.copy(xmin, x);
  int imin = 0, jmin = 0;
  double tolb = tol * n2b;
  g.copy(xm, x);
  int evalxm = 0, stag = 0, moresteps = 0;
  const int maxmsteps = std::min(std::min(n / 50, 5), n - maxit);
  const int maxstagsteps = 3;
  int minupdated = 0;
  double normr;
  if (x0_zero) {
    g.copy(r, b);
    normr = n2b;
  } else {
    g.residual(b, x, r);
    normr = g.norm(r);
  }
  if (g.rc) return g.rc;
  if (normr <= tolb) {
    *flag_out = 0; *relres_out = normr / n2b; iter_out[0] = iter_out[1] = 0;
    resvec_out.assign(1, normr);
    return PEEC_OK;
  }
  const double n2minv_b = n2b;
  tolb = tol * n2minv_b;
  std::vector<double> resvec((size_t)inner * outer + 1, 0.0);
  resvec[0] = normr;
  double normrmin = normr;
  const int ld = inner + 1;
  std::vector<cd> R((size_t)inner * inner), wv(inner + 1);
  std::vector<cd> Utop((size_t)ld * ld);
  int outitercount = 0, initercount = 0;
  double normr_act = normr;
  int it0 = 0, it1 = 0;
  const int headlen = (int)std::min<size_t>(N, (size_t)ld);
  // the cycle's device state and the buffers of the device loop's body
  CTX_TRY(ensure_gm(ctx, inner));
  const GmLayout GL = gm_layout(inner);
  unsigned char* gblk = ctx->gm_block;
  GmDev hdr = {};
  hdr.inner = inner;
  hdr.n = n;
  hdr.headlen = headlen;
  hdr.ld = ld;
  hdr.tolb = tolb;
  hdr.res = (double*)(gblk + GL.res);
  hdr.wv = (c64*)(gblk + GL.wv);
  hdr.J = (c64*)(gblk + GL.J);
  hdr.Utop = (c64*)(gblk + GL.Utop);
  hdr.R = (c64*)(gblk + GL.R);
  GmBody B;
  if (f32) B.U32 = ctx->U32;
  else B.U = ctx->U;
  B.N = N;
  B.T = ctx->dT;
  B.ldT = ldT;
  B.kmax = inner;
  B.gs = (GmDev*)gblk;
  B.v = v;
  B.w = add;
  B.coef = ctx->dcoef;
  B.coef2 = ctx->dcoef2;
  B.part = ctx->dpart;
  B.red = ctx->dred;
  B.scal = ctx->dscal;
  B.st = ctx->st;
  // the first k columns of R and Utop, read back for the host's least-squares solves
  // (the convergence checks on the true residual and the end of a cycle)
  auto pull = [&](int k) -> int {
    if (k <= 0) return PEEC_OK;
    cudaMemcpyAsync(Utop.data(), hdr.Utop, sizeof(c64) * (size_t)k * ld, cudaMemcpyDeviceToHost,
                    ctx->st);
    cudaMemcpyAsync(R.data(), hdr.R, sizeof(c64) * (size_t)k * inner, cudaMemcpyDeviceToHost,
                    ctx->st);
    PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
    return PEEC_OK;
  };
  for (int outiter = 1; outiter <= outer; ++outiter) {
    outitercount++;
    std::fill(Utop.begin(), Utop.end(), cd(0));
    PEEC_CUDA_TRY(cudaMemsetAsync(ctx->dT, 0, sizeof(c64) * (size_t)ldT * ldT, ctx->st));
    // u = r + sign(r1)*norm(r)*e1, normalised (later restart cycles use the true
    // residual norm of the end-of-cycle residual)
    if (outiter > 1) normr = g.norm(r);
    {
      const std::vector<cd> rh = g.from_dev(r, headlen);
      const cd beta = sgn(rh[0]) * normr;
      const double nu2 = normr * normr - std::norm(rh[0]) + std::norm(rh[0] + beta);
      const double sc = 1.0 / std::sqrt(nu2);
      if (f32)
        launch_make_reflector(r, N, 0, mk<double>(beta.real(), beta.imag()), sc, ctx->U32, ctx->st);
      else
        launch_make_reflector(r, N, 0, mk<double>(beta.real(), beta.imag()), sc, ctx->U, ctx->st);
      ctx->launches++;
      for (int i = 0; i < headlen; ++i) Utop[i] = (i == 0 ? rh[0] + beta : rh[i]) * sc;
      launch_tri(ctx->dT, ldT, 0, ctx->dcoef2, ctx->dT, 2, ctx->st);  // T(0,0) = 2
      ctx->launches++;
      wv.assign(inner + 1, cd(0));
      wv[0] = -beta;
      g.to_dev(hdr.Utop, std::vector<cd>(Utop.begin(), Utop.begin() + headlen));
      g.to_dev(hdr.wv, wv);
    }
    initercount = 0;
    int jdone = 0;       // iterations of this cycle done on the device
    bool leave = false;  // the cycle ended before its last iteration
    while (jdone < inner && !leave) {
      if (ctx->stop && *ctx->stop) {
        *flag_out = 99; *relres_out = 0; iter_out[0] = outiter; iter_out[1] = jdone + 1;
        resvec_out.assign(1, 0.0);
        return bad(ctx, PEEC_ERR_CANCELLED, "cancelled by stop flag");
      }
      // Iterations run on the device until the residual estimate reaches tolb, the cycle
      // is full, or (exit_now) the host's stagnation / extra-step logic wants each one.
      // Those that went on had none of the conditions of the check below, so only the
      // last one needs it: the reference's control flow, iteration for iteration.
      hdr.j = jdone;
      hdr.exit_now = (stag >= maxstagsteps || moresteps == 1) ? 1 : 0;
      hdr.normr = normr;
      std::memcpy(ctx->gm_up, &hdr, sizeof(GmDev));
      PEEC_CUDA_TRY(cudaMemcpyAsync(gblk, ctx->gm_up, sizeof(GmDev), cudaMemcpyHostToDevice,
                                    ctx->st));
      int64_t per_it = 0;
      CTX_TRY(gm_iterate(ctx, B, prec, inner, &per_it));
      PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->gm_down, gblk, GL.J, cudaMemcpyDeviceToHost, ctx->st));
      PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
      if (g.rc) return g.rc;
      const GmDev* hd = (const GmDev*)ctx->gm_down;
      const double* hres = (const double*)(ctx->gm_down + GL.res);
      const c64* hwv = (const c64*)(ctx->gm_down + GL.wv);
      const int jafter = hd->j;
      if (jafter <= jdone || jafter > inner)
        return bad(ctx, PEEC_ERR_CUDA, "device Arnoldi loop: the iteration count did not advance");
      if (per_it) {
        ctx->launches += per_it * (jafter - jdone);
        ctx->kg_iterations += jafter - jdone;
      }
      for (int i = 0; i <= inner; ++i) wv[i] = cd(hwv[i].x, hwv[i].y);
      for (int initer = jdone + 1; initer <= jafter; ++initer) {
        initercount++;
        const int j = initer - 1;
        normr = hres[initer];
        resvec[(size_t)(outiter - 1) * inner + initer] = normr;
        normr_act = normr;
        if (initer == jafter && (normr <= tolb || stag >= maxstagsteps || moresteps == 1)) {
          CTX_TRY(pull(initer));
          do {
            if (evalxm == 0) {
              std::vector<cd> rhs(wv.begin(), wv.begin() + initer);
              std::vector<cd> ytmp = utri_solve(R, inner, initer, rhs);
              apply_Q(g, Utop, ld, initer, ytmp, nullptr, add);
              const double na = g.norm(add), nx = g.norm(x);
              if (na < 2.220446049250313e-16 * nx) stag++;
              else stag = 0;
              // xm = x + additive
              apply_Q(g, Utop, ld, initer, ytmp, x, xm);
              evalxm = 1;
            } else {
              const cd wr = wv[j] / R[(size_t)j * inner + j];
              std::vector<cd> addvc(initer);
              if (initer > 1) {
                std::vector<cd> rhs(initer - 1);
                for (int i = 0; i < initer - 1; ++i) rhs[i] = R[(size_t)j * inner + i];
                std::vector<cd> hsol = utri_solve(R, inner, initer - 1, rhs);
                for (int i = 0; i < initer - 1; ++i) addvc[i] = -hsol[i] * wr;
              }
              addvc[initer - 1] = wr;
              double nav = 0;
              for (auto& q : addvc) nav += std::norm(q);
              nav = std::sqrt(nav);
              const double nxm = g.norm(xm);
              if (nav < 2.220446049250313e-16 * nxm) stag++;
              else stag = 0;
              g.copy(ctx->gtmp, xm);
              apply_Q(g, Utop, ld, initer, addvc, ctx->gtmp, xm);
            }
            g.residual(b, xm, r);
            const double nr = g.norm(r);
            if (g.rc) return g.rc;
            if (nr <= tol * n2b) {
              g.copy(x, xm);
              flag = 0;
              it0 = outiter;
              it1 = initer;
              leave = true;
              break;
            }
            normr_act = nr;
            resvec[(size_t)(outiter - 1) * inner + initer] = normr_act;
            if (normr_act <= normrmin) {
              normrmin = normr_act;
              imin = outiter;
              jmin = initer;
              g.copy(xmin, xm);
              minupdated = 1;
            }
            if (normr_act <= tolb) {
              g.copy(x, xm);
              flag = 0;
              it0 = outiter;
              it1 = initer;
              leave = true;
              break;
            } else {
              if (stag >= maxstagsteps && moresteps == 0) stag = 0;
              moresteps++;
              if (moresteps >= maxmsteps) {
                flag = 3;
                it0 = outiter;
                it1 = initer;
                leave = true;
                break;
              }
            }
          } while (false);
          if (leave) break;
        }
        if (normr_act <= normrmin) {
          normrmin = normr_act;
          imin = outiter;
          jmin = initer;
          minupdated = 1;
        }
        if (stag >= maxstagsteps) {
          flag = 3;
          leave = true;
          break;
        }
      }
      jdone = jafter;
    }
    evalxm = 0;
    if (flag != 0) {
      const int idx = minupdated == 1 ? jmin : initercount;
      if (idx > 0) {
        CTX_TRY(pull(idx));
        std::vector<cd> rhs(wv.begin(), wv.begin() + idx);
        std::vector<cd> y = utri_solve(R, inner, idx, rhs);
        g.copy(ctx->gtmp, x);
        apply_Q(g, Utop, ld, idx, y, ctx->gtmp, x);
      }
      g.copy(xmin, x);
      g.residual(b, x, r);
      normr_act = g.norm(r);
      if (g.rc) return g.rc;
    }
    if (normr_act <= normrmin) {
      g.copy(xmin, x);
      normrmin = normr_act;
      imin = outiter;
      jmin = initercount;
    }
    if (flag == 3) break;
    if (normr_act <= tolb) {
      flag = 0;
      it0 = outitercount;
      it1 = initercount;
      break;
    }
    minupdated = 0;
  }
  double relres;
  if (flag == 0) {
    relres = normr_act / n2minv_b;
    g.copy(x_dev, x);
  } else {
    g.copy(x_dev, xmin);
    it0 = imin;
    it1 = jmin;
    relres = normr_act / n2minv_b;
  }
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  const size_t nres = (size_t)std::max(outitercount - 1, 0) * inner + initercount + 1;
  resvec_out.assign(resvec.begin(), resvec.begin() + std::min(nres, resvec.size()));
  *flag_out = flag;
  *relres_out = relres;
  iter_out[0] = it0;
  iter_out[1] = it1;
  return g.rc;
}

static int peec_gmres_body(peec_ctx* ctx, const double* b, double* x_inout, double tol, int maxit,
                          int restarted, int restart, int precision, int* flag, double* relres,
                          int* iter, double* resvec, int resvec_cap, int* nres) {
  NvtxRange nvtx_range_("peec_gmres");
  if (!ctx || !b || !x_inout || !flag || !relres || !iter) return badarg("peec_gmres");
  if (maxit < 1 || (restarted && restart < 1)) return bad(ctx, PEEC_ERR_BADARG, "maxit/restart must be >= 1");
  if (precision < 0 || precision > 2) return bad(ctx, PEEC_ERR_BADARG, "precision must be 0, 1 or 2");
  if (!ctx->have_freq) return bad(ctx, PEEC_ERR_STATE, "frequency state not set");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const size_t bytes = sizeof(c64) * ctx->N;
  PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->dx, b, bytes, cudaMemcpyHostToDevice, ctx->st));
  PEEC_CUDA_TRY(cudaMemcpyAsync(ctx->dy, x_inout, bytes, cudaMemcpyHostToDevice, ctx->st));
  std::vector<double> rv;
  int rc = gmres_run(ctx, ctx->dx, ctx->dy, tol, maxit, restarted, restart, precision, flag,
                     relres, iter, rv);
  if (rc != PEEC_OK && rc != PEEC_ERR_CANCELLED) return rc;
  if (rc == PEEC_OK)
    PEEC_CUDA_TRY(cudaMemcpyAsync(x_inout, ctx->dy, bytes, cudaMemcpyDeviceToHost, ctx->st));
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  if (nres) *nres = (int)rv.size();
  if (resvec)
    for (int i = 0; i < (int)rv.size() && i < resvec_cap; ++i) resvec[i] = rv[i];
  if (rc == PEEC_ERR_CANCELLED) ctx->err = "cancelled by stop flag";
  else CTX_TRY(check_solve_errors(ctx));
  return rc;
}

static int peec_solve_mixed_body(peec_ctx* ctx, const double* b, double* x_inout, double tol,
                                double inner_tol, int inner_maxit, int max_outer, int* flag,
                                double* relres, int* outer_out, int* inner_total) {
  NvtxRange nvtx_range_("peec_solve_mixed");
  if (!ctx || !b || !x_inout || !flag || !relres) return badarg("peec_solve_mixed");
  if (!ctx->have_freq) return bad(ctx, PEEC_ERR_STATE, "frequency state not set");
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  const size_t N = ctx->N, bytes = sizeof(c64) * N;
  c64 *db = ctx->ir_b, *dxv = ctx->ir_x, *dr = ctx->ir_r, *dd = ctx->ir_d;
  auto cleanup = [&]() {};
  CTX_TRY(ensure_krylov(ctx, std::max(inner_maxit, 1) + 1, PEEC_PREC_FP32));
  cudaMemcpyAsync(db, b, bytes, cudaMemcpyHostToDevice, ctx->st);
  cudaMemcpyAsync(dxv, x_inout, bytes, cudaMemcpyHostToDevice, ctx->st);
  Gm g{ctx, N, ctx->resid_prec, ctx->st};
  // The convolutions Lp*I and P*Q do not depend on the frequency. When x0 is the solution
  // this context returned last (the warm start of a frequency sweep), the first residual
  // reuses the convolutions of that solve's final residual -- the same numbers a fresh
  // application would produce -- and only the sparse half runs.
  bool reuse = false;
  if (ctx->cc_prec == ctx->resid_prec) {
    cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->st);
    launch_differs(dxv, ctx->cc_x, N, ctx->d_flag, ctx->st);
    ctx->launches++;
    cudaMemcpyAsync(ctx->hscal, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->st);
    PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
    reuse = *(const int*)ctx->hscal == 0;
  }
  ctx->cc_prec = -1;  // re-armed below once this solve converges
  bool fresh = false;  // the last residual computed its own convolutions
  const double n2b = g.norm(db);
  int outer = 0, tot_inner = 0, fl = 1;
  double rel = 0;
  if (n2b == 0) {
    cudaMemsetAsync(dxv, 0, bytes, ctx->st);
    fl = 0;
  } else {
    // a zero initial guess makes the first residual b itself (A*0 is exactly 0)
    const bool x_zero = g.norm(dxv) == 0.0;
    for (outer = 0; outer <= max_outer; ++outer) {
      double nr;
      if (outer == 0 && x_zero) {
        g.copy(dr, db);
        nr = n2b;
        fresh = false;
      } else if (outer == 0 && reuse) {
        sparse_enqueue(ctx, dxv, ctx->gtmp, ctx->cc_LpI, ctx->cc_PQ);
        launch_sub(db, ctx->gtmp, N, dr, ctx->st);
        ctx->launches++;
        nr = g.norm(dr);
        fresh = false;
      } else {
        g.residual(db, dxv, dr);  // FP64 or float-float operator
        nr = g.norm(dr);
        fresh = true;
      }
      if (g.rc) { cleanup(); return g.rc; }
      rel = nr / n2b;
      if (rel <= tol) { fl = 0; break; }
      if (outer == max_outer) break;
      if (ctx->stop && *ctx->stop) { cleanup(); ctx->err = g_err = "cancelled by stop flag"; *flag = 99; return PEEC_ERR_CANCELLED; }
      // inner correction on the FP32-convolution operator, zero initial guess. The inner
      // target leaves a 20% margin below what the outer tolerance needs (tol / rel
      // relative to this residual): the FP32 operator's own error, ~1e-7 of |A d|, adds
      // ~1e-7 * rel to the corrected residual, far below that margin for the warm-started
      // residuals (rel ~1e-2) of a sweep.
      cudaMemsetAsync(dd, 0, bytes, ctx->st);
      const double itol = std::max(inner_tol, 0.8 * tol / rel);
      int ifl, it[2];
      double irel;
      std::vector<double> rv;
      int rc = gmres_run(ctx, dr, dd, std::min(itol, 0.5), inner_maxit, 0, 0, 1, &ifl, &irel, it, rv,
                         true);
      if (rc) { cleanup(); return rc; }
      tot_inner += (int)rv.size() - 1;
      launch_add(dxv, dd, N, dxv, ctx->st);  // x += d
      ctx->launches++;
    }
  }
  if (fl == 0 && n2b != 0 && (fresh || reuse)) {
    // keep the convolutions of the returned solution for the next frequency's warm start
    if (fresh) {
      cudaMemcpyAsync(ctx->cc_x, dxv, bytes, cudaMemcpyDeviceToDevice, ctx->st);
      cudaMemcpyAsync(ctx->cc_LpI, ctx->LpI, sizeof(c64) * ctx->m, cudaMemcpyDeviceToDevice,
                      ctx->st);
      cudaMemcpyAsync(ctx->cc_PQ, ctx->PQ, sizeof(c64) * ctx->ns, cudaMemcpyDeviceToDevice,
                      ctx->st);
    }
    ctx->cc_prec = ctx->resid_prec;
  }
  cudaMemcpyAsync(x_inout, dxv, bytes, cudaMemcpyDeviceToHost, ctx->st);
  PEEC_CUDA_TRY(cudaStreamSynchronize(ctx->st));
  CTX_TRY(check_solve_errors(ctx));
  *flag = fl;
  *relres = rel;
  if (outer_out) *outer_out = outer;
  if (inner_total) *inner_total = tot_inner;
  return PEEC_OK;
}

static int peec_set_residual_precision_body(peec_ctx* ctx, int precision) {
  if (!ctx) return badarg("peec_set_residual_precision");
  if (precision != PEEC_PREC_FP64 && precision != PEEC_PREC_FF)
    return bad(ctx, PEEC_ERR_BADARG, "residual precision must be PEEC_PREC_FP64 or PEEC_PREC_FF");
  ctx->resid_prec = precision;
  return PEEC_OK;
}

static int peec_set_lu_component_max_body(peec_ctx* ctx, int max_rows) {
  if (!ctx) return badarg("peec_set_lu_component_max");
  if (max_rows < 0 || max_rows > SF_COMP_MAX)
    return bad(ctx, PEEC_ERR_BADARG, "component size limit outside 0.." + std::to_string(SF_COMP_MAX));
  PEEC_CUDA_TRY(cudaSetDevice(ctx->dev));
  drop_graphs(ctx);
  ctx->comp_max = max_rows;
  if (ctx->have_freq) CTX_TRY(build_solve_plan(ctx, ctx->n));
  return PEEC_OK;
}

// ---------------------------------------------------------------------------------------
// Exported entry points. Each runs its body under one guard, so that no C++ exception
// reaches the caller: an exhausted host allocation returns PEEC_ERR_OOM, any other
// exception PEEC_ERR_STATE, each with its message for peec_last_error.

static void record_exception(peec_ctx* ctx, const char* fn, const char* what) noexcept {
  try {
    std::string msg = std::string(fn) + ": " + what;
    g_err = msg;
    if (ctx) ctx->err = msg;
  } catch (...) {
    g_err.assign("out of memory");  // fits the string's inline buffer: no allocation
  }
}

template <typename F>
static int guarded(peec_ctx* ctx, const char* fn, F&& body) noexcept {
  DeviceRestore restore_device_;
  try {
    return body();
  } catch (const std::bad_alloc&) {
    record_exception(ctx, fn, "host memory allocation failed");
    return PEEC_ERR_OOM;
  } catch (const std::length_error& e) {
    record_exception(ctx, fn, e.what());
    return PEEC_ERR_OOM;
  } catch (const std::exception& e) {
    record_exception(ctx, fn, e.what());
    return PEEC_ERR_STATE;
  } catch (...) {
    record_exception(ctx, fn, "unknown exception");
    return PEEC_ERR_STATE;
  }
}

extern "C" int peec_ctx_create(peec_ctx** out, int device) {
  return guarded(nullptr, "peec_ctx_create", [&] {
    return peec_ctx_create_body(out, device);
  });
}

extern "C" int peec_set_topology(peec_ctx* ctx, int Nx, int Ny, int Nz, int64_t mx, int64_t my,
                                 int64_t mz, const int64_t* edge_cell, const int64_t* edge_n1,
                                 const int64_t* edge_n2, int64_t ns, const int32_t* surf_fam,
                                 const int64_t* surf_cell, const int64_t* surf_node, int64_t n) {
  return guarded(ctx, "peec_set_topology", [&] {
    return peec_set_topology_body(ctx, Nx, Ny, Nz, mx, my, mz, edge_cell, edge_n1, edge_n2, ns,
        surf_fam, surf_cell, surf_node, n);
  });
}

extern "C" int peec_set_incidence(peec_ctx* ctx, int64_t mx, int64_t my, int64_t mz,
                                  const int64_t* edge_n1, const int64_t* edge_n2, int64_t ns,
                                  const int64_t* surf_node, int64_t n) {
  return guarded(ctx, "peec_set_incidence", [&] {
    return peec_set_incidence_body(ctx, mx, my, mz, edge_n1, edge_n2, ns, surf_node, n);
  });
}

extern "C" int peec_set_dense(peec_ctx* ctx, const double* Lp_x, const double* Lp_y,
                              const double* Lp_z, const double* P) {
  return guarded(ctx, "peec_set_dense", [&] { return peec_set_dense_body(ctx, Lp_x, Lp_y, Lp_z, P); });
}

extern "C" int peec_ris_fill(peec_ctx* ctx, const double* vol_coords, const double* vol_S,
                             const double* vol_centres, double escal_Lp, const double* surf_ends,
                             const double* surf_S, const double* surf_centres, double escal_P,
                             int distances, int64_t* nonfinite) {
  return guarded(ctx, "peec_ris_fill", [&] {
    return peec_ris_fill_body(ctx, vol_coords, vol_S, vol_centres, escal_Lp, surf_ends, surf_S,
                              surf_centres, escal_P, distances, nonfinite);
  });
}

extern "C" int peec_dense_get(peec_ctx* ctx, int block, int what, double* out) {
  return guarded(ctx, "peec_dense_get", [&] { return peec_dense_get_body(ctx, block, what, out); });
}

extern "C" int peec_set_edge_state(peec_ctx* ctx, const double* R4, const double* Cd4,
                                   const double* Lp_self, const double* Zs0,
                                   const int64_t* surface_edges, int64_t nse, double escal_R,
                                   double escal_freq) {
  return guarded(ctx, "peec_set_edge_state", [&] {
    return peec_set_edge_state_body(ctx, R4, Cd4, Lp_self, Zs0, surface_edges, nse, escal_R,
                                    escal_freq);
  });
}

extern "C" int peec_set_frequency_device(peec_ctx* ctx, double w, int64_t yle_nnz,
                                         const int64_t* yle_row, const int64_t* yle_col,
                                         const double* yle_val) {
  return guarded(ctx, "peec_set_frequency_device", [&] {
    return peec_set_frequency_device_body(ctx, w, yle_nnz, yle_row, yle_col, yle_val);
  });
}

extern "C" int peec_set_dense_rcc(peec_ctx* ctx, const double* Rx, const double* Ry,
                                  const double* Rz, const double* Rcc) {
  return guarded(ctx, "peec_set_dense_rcc", [&] { return peec_set_dense_rcc_body(ctx, Rx, Ry, Rz, Rcc); });
}

extern "C" int peec_set_dense_rcc_frequency(peec_ctx* ctx, double beta) {
  return guarded(ctx, "peec_set_dense_rcc_frequency",
                 [&] { return peec_set_dense_rcc_frequency_body(ctx, beta); });
}

extern "C" int peec_set_pdiag(peec_ctx* ctx, const double* diagP) {
  return guarded(ctx, "peec_set_pdiag", [&] {
    return peec_set_pdiag_body(ctx, diagP);
  });
}

extern "C" int peec_set_rows(peec_ctx* ctx, const double* const rows[9]) {
  return guarded(ctx, "peec_set_rows", [&] {
    return peec_set_rows_body(ctx, rows);
  });
}

extern "C" int peec_fill(peec_ctx* ctx, const double origin[3], double sx, double sy, double sz,
                         double escal_Lp, double escal_P, double* const rows_out[9]) {
  return guarded(ctx, "peec_fill", [&] {
    return peec_fill_body(ctx, origin, sx, sy, sz, escal_Lp, escal_P, rows_out);
  });
}

extern "C" int peec_fill_rcc(peec_ctx* ctx, const double origin[3], double sx, double sy,
                             double sz, double escal_Lp, double escal_P, double* const rows_out[9]) {
  return guarded(ctx, __func__, [&] {
    return peec_fill_rcc_body(ctx, origin, sx, sy, sz, escal_Lp, escal_P, rows_out);
  });
}

extern "C" int peec_set_rows_rcc(peec_ctx* ctx, const double* const rows[9],
                                 const double origin[3], double sx, double sy, double sz) {
  return guarded(ctx, __func__,
                 [&] { return peec_set_rows_rcc_body(ctx, rows, origin, sx, sy, sz); });
}

extern "C" int peec_set_rcc_frequency(peec_ctx* ctx, double freq_hz) {
  return guarded(ctx, __func__, [&] { return peec_set_rcc_frequency_body(ctx, freq_hz); });
}

extern "C" int peec_lu_refactor_setup(peec_ctx* ctx, int64_t yle_nnz, const int64_t* yle_row,
                                      const int64_t* yle_col) {
  return guarded(ctx, "peec_lu_refactor_setup",
                 [&] { return peec_lu_refactor_setup_body(ctx, yle_nnz, yle_row, yle_col); });
}

extern "C" int peec_set_frequency_refactor(peec_ctx* ctx, double w, const double* DZ,
                                           int64_t yle_nnz, const int64_t* yle_row,
                                           const int64_t* yle_col, const double* yle_val) {
  return guarded(ctx, "peec_set_frequency_refactor", [&] {
    return peec_set_frequency_refactor_body(ctx, w, DZ, yle_nnz, yle_row, yle_col, yle_val);
  });
}

extern "C" int peec_set_frequency(peec_ctx* ctx, double w, const double* DZ, int64_t yle_nnz,
                                  const int64_t* yle_row, const int64_t* yle_col,
                                  const double* yle_val, const int64_t* L_ptr,
                                  const int64_t* L_col, const double* L_val,
                                  const int64_t* U_ptr, const int64_t* U_col,
                                  const double* U_val, const int64_t* perm_r,
                                  const int64_t* perm_c, const double* row_scale) {
  return guarded(ctx, "peec_set_frequency", [&] {
    return peec_set_frequency_body(ctx, w, DZ, yle_nnz, yle_row, yle_col, yle_val, L_ptr, L_col,
        L_val, U_ptr, U_col, U_val, perm_r, perm_c, row_scale);
  });
}

extern "C" int peec_matvec_dev(peec_ctx* ctx, const void* x, void* y, int precision) {
  return guarded(ctx, "peec_matvec_dev", [&] {
    return peec_matvec_dev_body(ctx, x, y, precision);
  });
}

extern "C" int peec_matvec(peec_ctx* ctx, const double* x, double* y, int precision) {
  return guarded(ctx, "peec_matvec", [&] {
    return peec_matvec_body(ctx, x, y, precision);
  });
}

extern "C" int peec_profile_matvec(peec_ctx* ctx, int precision, int iters, double* ms) {
  return guarded(ctx, "peec_profile_matvec", [&] {
    return peec_profile_matvec_body(ctx, precision, iters, ms);
  });
}

extern "C" int peec_multidot(peec_ctx* ctx, const void* U, int64_t ldu, const void* v, int64_t N,
                             int k, void* out) {
  return guarded(ctx, "peec_multidot", [&] {
    return peec_multidot_body(ctx, U, ldu, v, N, k, out);
  });
}

extern "C" int peec_port_rhs(peec_ctx* ctx, int64_t n1, int64_t n2, double Is, double* tn) {
  return guarded(ctx, "peec_port_rhs", [&] {
    return peec_port_rhs_body(ctx, n1, n2, Is, tn);
  });
}

extern "C" int peec_check_wait_limit(peec_ctx* ctx) {
  return guarded(ctx, "peec_check_wait_limit", [&] {
    return peec_check_wait_limit_body(ctx);
  });
}

extern "C" int peec_adjoint(peec_ctx* ctx, const double* x, const int32_t* v1,
                            const int32_t* v2, const double* d1, const double* d2, double Is,
                            int64_t nvox, double* g) {
  return guarded(ctx, "peec_adjoint", [&] {
    return peec_adjoint_body(ctx, x, v1, v2, d1, d2, Is, nvox, g);
  });
}

extern "C" int peec_gmres(peec_ctx* ctx, const double* b, double* x_inout, double tol, int maxit,
                          int restarted, int restart, int precision, int* flag, double* relres,
                          int* iter, double* resvec, int resvec_cap, int* nres) {
  return guarded(ctx, "peec_gmres", [&] {
    return peec_gmres_body(ctx, b, x_inout, tol, maxit, restarted, restart, precision, flag,
        relres, iter, resvec, resvec_cap, nres);
  });
}

extern "C" int peec_solve_mixed(peec_ctx* ctx, const double* b, double* x_inout, double tol,
                                double inner_tol, int inner_maxit, int max_outer, int* flag,
                                double* relres, int* outer_out, int* inner_total) {
  return guarded(ctx, "peec_solve_mixed", [&] {
    return peec_solve_mixed_body(ctx, b, x_inout, tol, inner_tol, inner_maxit, max_outer, flag,
        relres, outer_out, inner_total);
  });
}

extern "C" int peec_set_lu_component_max(peec_ctx* ctx, int max_rows) {
  return guarded(ctx, "peec_set_lu_component_max", [&] {
    return peec_set_lu_component_max_body(ctx, max_rows);
  });
}

extern "C" int peec_set_residual_precision(peec_ctx* ctx, int precision) {
  return guarded(ctx, "peec_set_residual_precision", [&] {
    return peec_set_residual_precision_body(ctx, precision);
  });
}
