// Internal declarations shared by the translation units of libpeec_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "common.cuh"

namespace peec {

int fail_cuda(cudaError_t e, const char* expr, const char* file, int line);
void set_error(const std::string& msg);

#define PEEC_ERR_UNSUPPORTED_INTERNAL (-6)

// one triangle of the synchronisation-free LU solve (CSR without the diagonal)
struct SfTri {
  const int32_t* ptr;
  const int32_t* col;
  const c64* val;
  const c64* dinv;
  int* flag;  // per row: the epoch of the solve that last finished the row
};
constexpr int SF_TPB = 128;

// Groups of the LU solves (sparse.cu, k_sptrsv_grp). The rows of L and U fall into
// connected components (rows linked by a factor entry) that never depend on one another.
// Components of at most 32 rows (and SF_GRP_E entries) are packed into groups of at most
// 32 rows; larger ones (up to SF_COMP_MAX rows) form a group each. One warp solves a
// group: it loads all of the group's rows, entries and right-hand sides into shared
// memory with parallel loads, then runs the group's L levels and U levels there.
constexpr int SF_COMP_MAX = 512;
constexpr int SF_GRP_E = 256;  // entries (L and U off-diagonal) of a packed group
constexpr int SF_GRP_WARPS = 4;
constexpr int SF_BIG_LANES = 4;  // lanes per row in the large components' level loops
struct GrpRow {
  int32_t r;       // factor row
  int32_t pL, pU;  // first entry of the row in L and in U (CSR)
  int32_t j;       // original row of its right-hand side (Pr)
  int16_t nL, nU;  // entries of the row in L and in U
  int16_t eL, eU;  // their offsets in the group's shared entry array
};
struct GrpPlan {
  const int32_t* goff = nullptr;    // ngroups + 1 offsets into rows
  const GrpRow* rows = nullptr;     // per position: the group's rows in L-level order
  const int16_t* uq = nullptr;      // per position in U-level order: that row's L position
  const int32_t* seg = nullptr;     // per group: ends of its L levels, then of its U levels
  const int32_t* segoff = nullptr;  // ngroups + 1 offsets into seg
  const int32_t* nsegL = nullptr;   // per group: the number of its L level ends
  const int16_t* lcolL = nullptr;   // per L entry (CSR order): its column's L position
  const int16_t* lcolU = nullptr;   // per U entry
  int nbig = 0, ngroups = 0;        // groups [0, nbig) hold one large component each
  int rb = 0, eb = 0;               // the large groups' largest row and entry counts
};
// shared memory of one group of R rows and E entries
__host__ __device__ inline size_t grp_smem(int R, int E) {
  size_t o = 48 * (size_t)R + 16 * (size_t)E;  // x, 1/L(i,i), 1/U(i,i), entry values
  o += 8 * (size_t)R + 2 * (size_t)E + 2 * (size_t)R;  // row metadata, entry columns, U order
  o = (o + 3) & ~(size_t)3;
  o += 8 * (size_t)R;  // level ends (at most 2R)
  return (o + 15) & ~(size_t)15;
}

// Device refactorisation of SS in a fixed pattern (refactor.cu): slots are the off-diagonal
// entries of L, then the diagonal of U (D), then the off-diagonal entries of U
struct RefactorPlan {
  int64_t n = 0, nL = 0, nU = 0;
  int64_t* asm_ptr = nullptr;    // per slot, its contributions in asm_src
  uint32_t* asm_src = nullptr;   // contribution codes (type << 30 | index)
  int32_t* rows = nullptr;       // rows grouped by L level
  std::vector<int> lvl_off;      // level offsets into rows (host)
  int32_t* upd_off = nullptr;    // per L entry (p, k): its targets in upd_tgt
  int32_t* upd_tgt = nullptr;    // per entry of U(k,:): its slot in row p
  c64* D = nullptr;              // diagonal of U
};
int refactor_launch(const RefactorPlan& R, const SfTri& L, const SfTri& U, c64* Lval, c64* Uval,
                    const c64* DZ, const double* invP, const c64* yle, double w, int* err,
                    cudaStream_t st);

// Device-resident state of one Householder GMRES cycle (the Arnoldi loop's scalar work
// runs in k_gm_step, krylov.cu). The host writes the header before a run of iterations
// and reads back the header, res and wv after it; Utop and R only when its convergence
// check needs them. All arrays live in one allocation after the header.
struct GmDev {
  int j;          // inner iterations done in this cycle (the next one's 0-based index)
  int inner;      // iterations per cycle
  int n;          // system size (the reference's initer != n tests)
  int headlen;    // min(N, inner + 1): rows of the reflectors kept in Utop
  int ld;         // inner + 1, leading dimension of Utop
  int exit_now;   // host: leave the loop after the next iteration
  int refl_on;    // the last iteration appended a reflector (alpha != 0)
  int pad_;
  double tolb;    // tol * |b|: the loop continues while |w(j+1)| > tolb
  double normr;   // |w(j+1)| after the last iteration
  double refl_scale;
  double pad2_;
  c64 refl_add;   // the new reflector: u = (v with rows < j zeroed, v(j) += add) * scale
  double* res;    // [inner + 2] residual estimates, res[initer] = |w(initer)|
  c64* wv;        // [inner + 1] Givens-rotated right-hand side w
  c64* J;         // [2 * inner] Givens rotations (c, s) per column
  c64* Utop;      // [ld * ld] leading rows of the reflectors, column-major
  c64* R;         // [inner * inner] upper-triangular R, column-major, ld = inner
};

// Buffers of the device loop's Arnoldi body (krylov.cu): the basis is U (complex double)
// or U32 (complex float-float), whichever is set; T the compact-WY factor (ld ldT); v the
// iteration's vector, w = A v; kmax the largest column count of the cycle (inner).
struct GmBody {
  c64* U = nullptr;
  cff* U32 = nullptr;
  size_t N = 0;
  c64* T = nullptr;
  int ldT = 0, kmax = 0;
  GmDev* gs = nullptr;
  c64 *v = nullptr, *w = nullptr, *coef = nullptr, *coef2 = nullptr, *part = nullptr;
  double *red = nullptr, *scal = nullptr;
  cudaGraphConditionalHandle cond = 0;
  int use_cond = 0;  // 1 inside the WHILE node's body graph, 0 for a single eager iteration
  cudaStream_t st = nullptr;
};
int gm_pre(const GmBody& B);   // returns the kernels launched
int gm_post(const GmBody& B);

#define CTX_CHECK(expr)      \
  do {                       \
    int _r = (expr);         \
    if (_r) return _r;       \
  } while (0)

// A lattice family: one face family of the P tensor (reference families 12, 34, 56)
// or one edge direction of the Lp tensor. Its lattice is both the input and the
// output lattice of its circulant blocks.
struct Family {
  bool active = false;
  bool lp = false;       // edge family (compact vector I, output LpI) vs face family (Q, PQ)
  int dims[3] = {0, 0, 0};  // lattice extents, x fastest
  int L[3] = {1, 1, 1}, logL[3] = {0, 0, 0};  // circulant grid
  int32_t* map = nullptr;   // lattice cell -> compact index or -1
  void* T[2] = {nullptr, nullptr};  // work buffer per precision: [z < dims[2]][y < Ly][kx < Lx]
};

// A block spectrum, scaled by 1/(Lx*Ly*Lz), in two forms.
// Full: every position, layout (ky, kz, kx), kx fastest, in the transforms' bit-reversed
//   position order; real for symmetric kernels; FP64 and FP32 copies (coalesced reads for
//   the FP32 and FP64 passes).
// Octant: along each axis the kernel is even (c = 0) or even about a half-sample shift
//   (c = +-1), so S(k) = R(|k_x|, |k_y|, |k_z|) * prod_a exp(-i*pi*c_a*k_a/L_a) with
//   k_a in (-L_a/2, L_a/2] and R real; the (L_x/2+1)(L_y/2+1)(L_z/2+1) values of R are kept
//   in FP64, layout (fy, fz, fx), fx fastest. The float-float passes read this form: an
//   eighth (a sixteenth for cross blocks) of the FP64 bytes.
// y/z-folded FP32 form (the FP32 z passes): R at the folded y and z frequencies but at
//   every x position, layout (fy, fz, px), px the DIF position, so a z-pass tile's 16
//   consecutive columns read 64 contiguous bytes; Lx(Ly/2+1)(Lz/2+1) floats, about a
//   quarter of the full FP32 form. Cross blocks take their half-sample phases at run time
//   from the FP32 phase tables.
struct Spectrum {
  int L[3] = {1, 1, 1};
  int c[3] = {0, 0, 0};
  int is_complex = 0;
  void* d[2] = {nullptr, nullptr};  // full: [0] fp64, [1] fp32
  void* oct = nullptr;              // octant R, fp64
  void* yz32 = nullptr;             // y/z-folded R, fp32
};

// Launchers (fftconv.cu). prec: 0 = fp64, 1 = fp32, 2 = float-float; tw[prec] the master
// twiddle table of that arithmetic. x (input) / LpI / PQ are complex double; families
// 0..2 are the face families, 3..5 the edge families; spectra 0..5 = P blocks
// (00, 11, 22, 01, 02, 12), 6..8 = Lp blocks of families 3..5.
// FP32 z-pass forms, chosen per grid by measurement (tune_zpass in ctx.cu). Face / edge
// form 0: register-direct kernels on the full-form spectra; 1: register-direct kernels on
// the y/z-folded spectra; 2: staged kernels (persistent CTAs, bulk-copied tiles, y/z-folded
// spectra; the edge families in one launch). edge_plan: the edge families' z radix plan
// (0: make_plan(n, 4, 4, 4), 1: make_plan(n, 4, 4, 3); 8 x 16 and 16 x 8 at Lz = 128).
struct ZTune {
  int* err = nullptr;  // error word set by a staged kernel whose copy wait ran into its limit
  int nsm = 0;         // SM count of the device
  int face = 0, edge = 0, edge_plan = 0;
};
// ev (nullable): 6 events around the five pass classes. ph: the face grid's phase tables,
// FP64 (x, y, z) then FP32 (x, y, z). zt (nullable: form 0): the FP32 z-pass choice.
int conv_all(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
             const c64* x, c64* LpI, c64* PQ, int64_t m, int prec, const void* const* tw,
             int twmax, cudaStream_t st, cudaEvent_t* ev, const ZTune* zt);
// one FP32 z pass alone, in the forms of zt (which 0: the face families, 1: the edge
// families), on the current family buffers; the tuner times it
int zpass_f32(const Family* F, int nfam, const Spectrum* spec, const void* const* ph,
              const void* tw, int twmax, const ZTune& zt, int which, cudaStream_t st);
// phase tables exp(-i*pi*k/L) per DIF position of the three face-grid axes, complex FP64
// (e64) and FP32 (e32)
int phase_tables(const int L[3], void* e64[3], void* e32[3], cudaStream_t st);
// whether the face / edge families' FP32 z passes can take forms 1 and 2 (whole 16-column
// tiles, enough z points; the edge families on one shared grid)
bool zpass_yz_faces(const Family* F, int nfam);
bool zpass_yz_edges(const Family* F, int nfam);
int spectrum_build(Spectrum& S, const double* d_row, const int M[3], const int na[3],
                   const int nb[3], const int sdim[3], const int odim[3], int symmetric,
                   const void* twiddles64, int twmax, cudaStream_t st);

}  // namespace peec
