// Block-sparse epilogue of the PEEC operator and its block preconditioner.
//
// After the convolutions have produced LpI = Lp*I (per edge) and PQ = P*Q (per
// surface), the operator rows of compute_Matrix_vector_fft.jl:29-77 are
//   Y1 = jw*LpI + DZ.*I + A*Phi,   Y2 = PQ - Gamma'*Phi,
//   Y3 = -A'*I + Yle*Phi + jw*Gamma*Q,
// and the preconditioner (precond_3_3_vector, :84-146) is applied with one sparse
// LU solve instead of three, using linearity of F\ :
//   M  = F \ (A'*invZ*Y1 - jw*Gamma*invP*Y2 + Y3)
//   y1 = invZ.*(Y1 - A*M),  y2 = invP.*(Y2 + Gamma'*M),  y3 = M.
// A has two entries per edge (-1 at n1, +1 at n2); Gamma one entry per surface.
// Node-side sums use host-built CSR lists (node -> edges, node -> surfaces).
#include <algorithm>
#include <mutex>

#include "ctx.hpp"

namespace peec {

__global__ void k_edge_rows(const c64* __restrict__ I, const c64* __restrict__ Phi,
                            const c64* __restrict__ LpI, const c64* __restrict__ DZ,
                            const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                            const double* __restrict__ wp, int m, c64* Y1, c64* U1) {
  const double w = *wp;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
    const c64 l = LpI[e], d = DZ[e], i = I[e];
    const c64 a = Phi[n2[e]] - Phi[n1[e]];
    // jw*l + d*i + a
    c64 y = mk<double>(-w * l.y, w * l.x) + d * i + a;
    Y1[e] = y;
    // y / d
    const double den = d.x * d.x + d.y * d.y;
    U1[e] = mk<double>((y.x * d.x + y.y * d.y) / den, (y.y * d.x - y.x * d.y) / den);
  }
}

__global__ void k_surf_rows(const c64* __restrict__ PQ, const c64* __restrict__ Phi,
                            const int32_t* __restrict__ snode, const double* __restrict__ invP,
                            int ns, c64* Y2, c64* U2) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
    const c64 y = PQ[s] - Phi[snode[s]];
    Y2[s] = y;
    U2[s] = cscale(y, invP[s]);
  }
}

// t[node] = sum_e A(e,node)*U1[e] - jw*sum_s U2[s] + Y3[node]
// Y3[node] = -sum_e A(e,node)*I[e] + (Yle*Phi)[node] + jw*sum_s Q[s]
__global__ void k_node_rows(const c64* __restrict__ I, const c64* __restrict__ Q,
                            const c64* __restrict__ Phi, const c64* __restrict__ U1,
                            const c64* __restrict__ U2, const int32_t* __restrict__ ne_ptr,
                            const int32_t* __restrict__ ne_idx, const int32_t* __restrict__ ns_ptr,
                            const int32_t* __restrict__ ns_idx, const int32_t* __restrict__ yle_ptr,
                            const int32_t* __restrict__ yle_col, const c64* __restrict__ yle_val,
                            const double* __restrict__ wp, int n, c64* t) {
  const double w = *wp;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    c64 au = mk<double>(0, 0), ai = mk<double>(0, 0);
    for (int p = ne_ptr[v]; p < ne_ptr[v + 1]; ++p) {
      const int code = ne_idx[p];  // edge index * 2 + (1 if A = +1 else 0)
      const int e = code >> 1;
      if (code & 1) {
        au = au + U1[e];
        ai = ai + I[e];
      } else {
        au = au - U1[e];
        ai = ai - I[e];
      }
    }
    c64 su = mk<double>(0, 0), sq = mk<double>(0, 0);
    for (int p = ns_ptr[v]; p < ns_ptr[v + 1]; ++p) {
      const int s = ns_idx[p];
      su = su + U2[s];
      sq = sq + Q[s];
    }
    c64 yp = mk<double>(0, 0);
    for (int p = yle_ptr[v]; p < yle_ptr[v + 1]; ++p) yp = yp + yle_val[p] * Phi[yle_col[p]];
    // jw*(sq - su)
    const c64 d = sq - su;
    t[v] = au - ai + yp + mk<double>(-w * d.y, w * d.x);
  }
}

__global__ void k_final_rows(const c64* __restrict__ Y1, const c64* __restrict__ Y2,
                             const c64* __restrict__ M, const c64* __restrict__ DZ,
                             const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                             const int32_t* __restrict__ snode, const double* __restrict__ invP,
                             int m, int ns, int n, c64* y) {
  const int total = m + ns + n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    if (i < m) {
      const c64 v = Y1[i] - (M[n2[i]] - M[n1[i]]);
      const c64 d = DZ[i];
      const double den = d.x * d.x + d.y * d.y;
      y[i] = mk<double>((v.x * d.x + v.y * d.y) / den, (v.y * d.x - v.x * d.y) / den);
    } else if (i < m + ns) {
      const int s = i - m;
      y[i] = cscale(Y2[s] + M[snode[s]], invP[s]);
    } else {
      y[i] = M[i - m - ns];
    }
  }
}

// ---------------------------------------------------------------------------------------
// sparse LU solve x = Pc * (U \ (L \ (Pr * (Rs .* b)))), both triangles in one launch,
// synchronisation-free: every row carries a ready flag (the solve's epoch once its value
// is final); a warp claims 32 rows of one level at a time from a global counter, in
// level order (all L levels, then all U levels), waits until the rows it depends on are
// flagged, and publishes its results with release stores. A row only ever waits on rows
// claimed before it, by warps that are already running, so the solve always progresses;
// every wait is bounded nonetheless (after the limit the kernel records an error in
// ctl[2] and stops waiting, and all later waits return at once).
// ---------------------------------------------------------------------------------------

__global__ void k_perm_gather(const c64* __restrict__ b, const int32_t* __restrict__ perm,
                              const double* __restrict__ rs, int n, c64* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int j = perm[i];
    out[i] = rs ? cscale(b[j], rs[j]) : b[j];
  }
}

__global__ void k_perm_scatter(const c64* __restrict__ z, const int32_t* __restrict__ perm, int n,
                               c64* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[perm[i]] = z[i];
}

// L2-coherent loads and stores of values other SMs publish during the same launch
__device__ __forceinline__ c64 ld_cg(const c64* p) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return mk<double>(v.x, v.y);
}
__device__ __forceinline__ void st_cg(c64* p, c64 v) {
  __stcg(reinterpret_cast<double2*>(p), make_double2(v.x, v.y));
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ctl[0] epoch, ctl[1] row claim counter, ctl[2] error flag, ctl[3] unused
__global__ void k_sptrsv_begin(int* ctl) {
  ctl[0] += 1;
  ctl[1] = 0;
  ctl[3] = 0;
}

// One warp per group (GrpPlan): components of the factors, several small ones packed
// together or one large one. The warp first brings everything the group's solve reads
// into its slice of shared memory -- per row the right-hand side (gathered through Pr
// and scaled by Rs), both inverse diagonals, its L and U entries with their columns as
// positions in the group -- with every row's loads independent of the others', so the
// whole group costs a few round trips to memory. Then the L levels, the U levels (in
// place: a U row reads its own L value and the U values of rows of earlier U levels),
// __syncwarp between levels, and the results go out to z. Per row the arithmetic is that
// of k_sptrsv (right-hand side, entries subtracted in row order, times the inverse
// diagonal). R, E: the shared-memory capacity of a warp's slice (rows, entries).
// W lanes per row in the level loops: 1 for the packed groups (short rows, one lane each);
// more for the large components, whose rows carry tens of entries on a chain of dozens
// of levels: the lanes of a row split its entries and combine their partial sums with a
// fixed shuffle tree (the same order on every run).
template <int W>
__global__ void k_sptrsv_grp(GrpPlan P, int g0, int g1, int R, int E, SfTri L, SfTri U,
                             const c64* __restrict__ b, const double* __restrict__ rs, c64* z) {
  extern __shared__ __align__(16) unsigned char grp_sm[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  unsigned char* base = grp_sm + (size_t)wib * grp_smem(R, E);
  c64* xs = reinterpret_cast<c64*>(base);
  c64* dl = xs + R;
  c64* du = dl + R;
  c64* ev = du + R;
  short4* meta = reinterpret_cast<short4*>(ev + E);  // (eL, nL, eU, nU)
  int16_t* ec = reinterpret_cast<int16_t*>(meta + R);
  int16_t* uqs = ec + E;
  int32_t* segs = reinterpret_cast<int32_t*>(
      (reinterpret_cast<uintptr_t>(uqs + R) + 3) & ~(uintptr_t)3);
  for (int g = g0 + blockIdx.x * wpb + wib; g < g1; g += gridDim.x * wpb) {
    const int q0 = P.goff[g], nr = P.goff[g + 1] - q0;
    const int s0 = P.segoff[g], ns = P.segoff[g + 1] - s0, nsl = P.nsegL[g];
    for (int q = lane; q < nr; q += 32) {
      const GrpRow pr = P.rows[q0 + q];
      xs[q] = rs ? cscale(b[pr.j], rs[pr.j]) : b[pr.j];
      dl[q] = L.dinv[pr.r];
      du[q] = U.dinv[pr.r];
      meta[q] = make_short4(pr.eL, pr.nL, pr.eU, pr.nU);
      for (int t = 0; t < pr.nL; ++t) {
        ev[pr.eL + t] = L.val[pr.pL + t];
        ec[pr.eL + t] = P.lcolL[pr.pL + t];
      }
      for (int t = 0; t < pr.nU; ++t) {
        ev[pr.eU + t] = U.val[pr.pU + t];
        ec[pr.eU + t] = P.lcolU[pr.pU + t];
      }
      uqs[q] = P.uq[q0 + q];
    }
    for (int t = lane; t < ns; t += 32) segs[t] = P.seg[s0 + t];
    __syncwarp();
    if constexpr (W == 1) {
      int prev = 0;
      for (int s = 0; s < nsl; ++s) {
        const int se = segs[s];
        for (int q = prev + lane; q < se; q += 32) {
          const short4 m = meta[q];
          c64 acc = xs[q];
          for (int t = 0; t < m.y; ++t) acc = acc - ev[m.x + t] * xs[ec[m.x + t]];
          xs[q] = acc * dl[q];
        }
        __syncwarp();
        prev = se;
      }
      prev = 0;
      for (int s = nsl; s < ns; ++s) {
        const int se = segs[s];
        for (int t = prev + lane; t < se; t += 32) {
          const int q = uqs[t];
          const short4 m = meta[q];
          c64 acc = xs[q];
          for (int e = 0; e < m.w; ++e) acc = acc - ev[m.z + e] * xs[ec[m.z + e]];
          xs[q] = acc * du[q];
        }
        __syncwarp();
        prev = se;
      }
    } else {
      constexpr int G = 32 / W;  // rows in flight per step
      const int sub = lane % W, grp = lane / W;
      int prev = 0;
      for (int s = 0; s < ns; ++s) {
        const bool upper = s >= nsl;
        const int se = segs[s];
        for (int t0 = prev; t0 < se; t0 += G) {  // warp-uniform: every lane shuffles
          const int t = t0 + grp;
          const bool valid = t < se;
          const int q = valid ? (upper ? (int)uqs[t] : t) : 0;
          c64 part = mk<double>(0, 0);
          if (valid) {
            const short4 m = meta[q];
            const int e0 = upper ? m.z : m.x, ne = upper ? m.w : m.y;
            for (int e = sub; e < ne; e += W) part = part + ev[e0 + e] * xs[ec[e0 + e]];
          }
#pragma unroll
          for (int o = W / 2; o > 0; o >>= 1) {
            part.x += __shfl_xor_sync(0xffffffffu, part.x, o, W);
            part.y += __shfl_xor_sync(0xffffffffu, part.y, o, W);
          }
          if (valid && sub == 0) xs[q] = (xs[q] - part) * (upper ? du[q] : dl[q]);
        }
        __syncwarp();
        prev = s + 1 == nsl ? 0 : se;
      }
    }
    for (int q = lane; q < nr; q += 32) z[P.rows[q0 + q].r] = xs[q];
    __syncwarp();
  }
}

__device__ __forceinline__ void sf_wait(const int* f, int epoch, int* err, int limit) {
  int it = 0;
  while (ld_acquire(f) != epoch) {
    ++it;
    if (it >= limit) {
      atomicExch(err, 1);
      return;
    }
    if ((it & 63) == 0) {
      if (*(volatile int*)err) return;
      __nanosleep(64);
    }
  }
}

constexpr int SF_CHUNK = 4;  // row entries whose column and value are held in registers

__global__ void __launch_bounds__(SF_TPB) k_sptrsv(const int32_t* __restrict__ ord, int nL,
                                                   int total, SfTri L, SfTri U,
                                                   const c64* __restrict__ b,
                                                   const int32_t* __restrict__ g_in,
                                                   const double* __restrict__ rs, c64* y,
                                                   c64* z, int* ctl, int limit) {
  const int lane = threadIdx.x & 31;
  const int epoch = ctl[0];
  int* err = ctl + 2;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(ctl + 1, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const int r = ord[base + lane];
    if (r >= 0) {
      // L rows: y = L \ (Pr b); U rows: z = U \ y. Separate outputs: a U row may finish
      // while an L row that reads the same index is still pending.
      const bool up = base >= nL;
      const SfTri& T = up ? U : L;
      c64* out = up ? z : y;
      // everything that does not depend on other rows is loaded before the first wait
      const int p0 = T.ptr[r], p1 = T.ptr[r + 1];
      const c64 dr = T.dinv[r];
      c64 acc;
      if (!up) {
        const int j = g_in[r];
        acc = rs ? cscale(b[j], rs[j]) : b[j];
      }
      int cc[SF_CHUNK];
      c64 vv[SF_CHUNK];
#pragma unroll
      for (int q = 0; q < SF_CHUNK; ++q) {
        if (p0 + q < p1) {
          cc[q] = T.col[p0 + q];
          vv[q] = T.val[p0 + q];
        }
      }
      if (up) {
        sf_wait(L.flag + r, epoch, err, limit);
        acc = ld_cg(y + r);
      }
      for (int p = p0; p < p1; p += SF_CHUNK) {
        if (p > p0) {
#pragma unroll
          for (int q = 0; q < SF_CHUNK; ++q) {
            if (p + q < p1) {
              cc[q] = T.col[p + q];
              vv[q] = T.val[p + q];
            }
          }
        }
#pragma unroll
        for (int q = 0; q < SF_CHUNK; ++q) {
          if (p + q < p1) {
            sf_wait(T.flag + cc[q], epoch, err, limit);
            acc = acc - vv[q] * ld_cg(out + cc[q]);
          }
        }
      }
      st_cg(out + r, acc * dr);
      st_release(T.flag + r, epoch);
    }
  }
}

static inline unsigned grid_for(long long n, int tpb = 256) {
  long long g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return (unsigned)g;
}

void launch_edge_rows(const c64* I, const c64* Phi, const c64* LpI, const c64* DZ,
                      const int32_t* n1, const int32_t* n2, const double* w, int m, c64* Y1,
                      c64* U1, cudaStream_t st) {
  if (m > 0) k_edge_rows<<<grid_for(m), 256, 0, st>>>(I, Phi, LpI, DZ, n1, n2, w, m, Y1, U1);
}
void launch_surf_rows(const c64* PQ, const c64* Phi, const int32_t* snode, const double* invP,
                      int ns, c64* Y2, c64* U2, cudaStream_t st) {
  if (ns > 0) k_surf_rows<<<grid_for(ns), 256, 0, st>>>(PQ, Phi, snode, invP, ns, Y2, U2);
}
void launch_node_rows(const c64* I, const c64* Q, const c64* Phi, const c64* U1, const c64* U2,
                      const int32_t* ne_ptr, const int32_t* ne_idx, const int32_t* ns_ptr,
                      const int32_t* ns_idx, const int32_t* yle_ptr, const int32_t* yle_col,
                      const c64* yle_val, const double* w, int n, c64* t, cudaStream_t st) {
  k_node_rows<<<grid_for(n), 256, 0, st>>>(I, Q, Phi, U1, U2, ne_ptr, ne_idx, ns_ptr, ns_idx,
                                           yle_ptr, yle_col, yle_val, w, n, t);
}
void launch_final_rows(const c64* Y1, const c64* Y2, const c64* M, const c64* DZ,
                       const int32_t* n1, const int32_t* n2, const int32_t* snode,
                       const double* invP, int m, int ns, int n, c64* y, cudaStream_t st) {
  k_final_rows<<<grid_for((long long)m + ns + n), 256, 0, st>>>(Y1, Y2, M, DZ, n1, n2, snode,
                                                               invP, m, ns, n, y);
}
void launch_perm_gather(const c64* b, const int32_t* perm, const double* rs, int n, c64* out,
                        cudaStream_t st) {
  k_perm_gather<<<grid_for(n), 256, 0, st>>>(b, perm, rs, n, out);
}
void launch_perm_scatter(const c64* z, const int32_t* perm, int n, c64* out, cudaStream_t st) {
  k_perm_scatter<<<grid_for(n), 256, 0, st>>>(z, perm, n, out);
}
// Raises the shared memory the group kernel may be launched with on the current device
// to at least smem_bytes (the default limit is 48 KB per block). The limit belongs to the
// kernel, not to a context, so it only ever grows: contexts of other geometries on the
// same device keep what their plans need.
int sptrsv_grp_prepare(size_t smem_bytes) {
  static std::mutex mu;
  static size_t granted[256] = {};
  int dev = 0;
  PEEC_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return fail_cuda(cudaErrorInvalidDevice, "device", __FILE__, __LINE__);
  std::lock_guard<std::mutex> lock(mu);
  // set every time (a re-created context starts from the default again)
  const size_t v = std::max(smem_bytes, granted[dev]);
  PEEC_CUDA_TRY(cudaFuncSetAttribute(k_sptrsv_grp<1>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v));
  PEEC_CUDA_TRY(cudaFuncSetAttribute(k_sptrsv_grp<SF_BIG_LANES>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)v));
  granted[dev] = v;
  return 0;
}

// returns the number of kernels launched
// The large groups go to st2 (forked from st with ev_fork, joined back with ev_join) so
// that they run beside the packed groups: the two launches are independent (different
// rows), and each is set by its own deepest groups' chain of levels. Under stream capture
// the fork and join become graph edges.
int launch_sptrsv(const GrpPlan& P, cudaStream_t st2, cudaEvent_t ev_fork, cudaEvent_t ev_join,
                  const int32_t* ord, int nL, int total, const SfTri& L, const SfTri& U,
                  const c64* b, const int32_t* g_in, const double* rs, c64* y, c64* z, int* ctl,
                  cudaStream_t st) {
  int launches = 0;
  const bool fork = st2 && P.nbig > 0 && P.ngroups > P.nbig;
  if (fork) {
    cudaEventRecord(ev_fork, st);
    cudaStreamWaitEvent(st2, ev_fork, 0);
  }
  if (P.nbig > 0) {  // one warp per large component, shared memory sized for the largest
    k_sptrsv_grp<SF_BIG_LANES><<<P.nbig, 32, grp_smem(P.rb, P.eb), fork ? st2 : st>>>(
        P, 0, P.nbig, P.rb, P.eb, L, U, b, rs, z);
    ++launches;
  }
  if (fork) cudaEventRecord(ev_join, st2);
  if (P.ngroups > P.nbig) {
    const int nsmall = P.ngroups - P.nbig;
    const int blocks = (nsmall + SF_GRP_WARPS - 1) / SF_GRP_WARPS;
    k_sptrsv_grp<1><<<blocks, 32 * SF_GRP_WARPS, SF_GRP_WARPS * grp_smem(32, SF_GRP_E), st>>>(
        P, P.nbig, P.ngroups, 32, SF_GRP_E, L, U, b, rs, z);
    ++launches;
  }
  if (fork) cudaStreamWaitEvent(st, ev_join, 0);
  if (total <= 0) return launches;
  k_sptrsv_begin<<<1, 1, 0, st>>>(ctl);
  launches += 2;
  // at most two CTAs (eight warps) per SM: warps that wait on earlier rows take issue
  // slots from kernels of other streams, and more warps do not shorten the chain of
  // levels (the widest level at 128x128x64 is about 1,400 warp batches)
  const int warps = (total + 31) / 32;
  int blocks = (warps + SF_TPB / 32 - 1) / (SF_TPB / 32);
  if (blocks > 152 * 2) blocks = 152 * 2;
  if (blocks < 1) blocks = 1;
  k_sptrsv<<<blocks, SF_TPB, 0, st>>>(ord, nL, total, L, U, b, g_in, rs, y, z, ctl,
                                        1 << 20);
  return launches;
}

// The bounded-wait failure path of k_sptrsv on a two-row lower triangle whose second row
// depends on the first, with only the second row in the claim order: the first row's
// flag is never set, so the dependency wait runs into `limit` polls, records the error
// word and returns. Returns the error word (1 when the wait gave up).
int selftest_wait_limit(int limit, cudaStream_t st, int* err_out) {
  struct Host {
    int32_t ptr[3] = {0, 0, 1};
    int32_t col[1] = {0};
    c64 val[1];
    c64 dinv[2];
    int32_t ord[32];
    c64 b[2];
    int32_t g_in[2] = {0, 1};
    int ctl[4] = {0, 0, 0, 0};
    int flag[2] = {0, 0};
  } h;
  h.val[0] = mk<double>(0.5, 0);
  h.dinv[0] = h.dinv[1] = mk<double>(1, 0);
  h.b[0] = h.b[1] = mk<double>(1, 0);
  h.ord[0] = 1;
  for (int i = 1; i < 32; ++i) h.ord[i] = -1;
  Host* d = nullptr;
  c64* yz = nullptr;
  PEEC_CUDA_TRY(cudaMalloc(&d, sizeof(Host)));
  if (cudaMalloc(&yz, 4 * sizeof(c64)) != cudaSuccess) {
    cudaFree(d);
    return fail_cuda(cudaErrorMemoryAllocation, "selftest buffers", __FILE__, __LINE__);
  }
  cudaMemcpyAsync(d, &h, sizeof(Host), cudaMemcpyHostToDevice, st);
  SfTri L{d->ptr, d->col, d->val, d->dinv, d->flag};
  SfTri U = L;
  k_sptrsv_begin<<<1, 1, 0, st>>>(d->ctl);
  k_sptrsv<<<1, SF_TPB, 0, st>>>(d->ord, 32, 32, L, U, d->b, d->g_in, nullptr, yz, yz + 2, d->ctl,
                                  limit);
  int e = 0;
  cudaMemcpyAsync(&e, d->ctl + 2, sizeof(int), cudaMemcpyDeviceToHost, st);
  const cudaError_t rc = cudaStreamSynchronize(st);
  cudaFree(d);
  cudaFree(yz);
  if (rc != cudaSuccess) return fail_cuda(rc, "selftest_wait_limit", __FILE__, __LINE__);
  *err_out = e;
  return 0;
}

}  // namespace peec
