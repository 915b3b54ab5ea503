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
#include "ctx.hpp"

namespace peec {

__global__ void k_edge_rows(const c64* __restrict__ I, const c64* __restrict__ Phi,
                            const c64* __restrict__ LpI, const c64* __restrict__ DZ,
                            const int32_t* __restrict__ n1, const int32_t* __restrict__ n2,
                            double w, int m, c64* Y1, c64* U1) {
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
                            double w, int n, c64* t) {
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
// sparse LU solve x = Pc * (U \ (L \ (Pr * (Rs .* b)))) with level-scheduled
// triangular sweeps; one launch per level, rows of a level independent.
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

// rows of one level: x[r] = (x[r] - sum_{j != r} T[r,j] x[j]) / T[r,r]
__global__ void k_trsv_level(const int32_t* __restrict__ rows, int nrows,
                             const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                             const c64* __restrict__ val, const c64* __restrict__ dinv, c64* x) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrows; t += gridDim.x * blockDim.x) {
    const int r = rows[t];
    c64 acc = x[r];
    for (int p = ptr[r]; p < ptr[r + 1]; ++p) acc = acc - val[p] * x[col[p]];
    x[r] = acc * dinv[r];
  }
}

// a run of consecutive small levels [l0, l1) in one CTA: levels in order, rows of a
// level spread over the block, __syncthreads() between levels makes each level's
// results visible to the next (no inter-block dependencies, no waiting)
__global__ void __launch_bounds__(1024) k_trsv_tail(const int32_t* __restrict__ rows,
                                                    const int32_t* __restrict__ lvl_off, int l0,
                                                    int l1, const int32_t* __restrict__ ptr,
                                                    const int32_t* __restrict__ col,
                                                    const c64* __restrict__ val,
                                                    const c64* __restrict__ dinv, c64* x) {
  for (int l = l0; l < l1; ++l) {
    const int a = lvl_off[l], b = lvl_off[l + 1];
    for (int t = a + threadIdx.x; t < b; t += blockDim.x) {
      const int r = rows[t];
      c64 acc = x[r];
      for (int p = ptr[r]; p < ptr[r + 1]; ++p) acc = acc - val[p] * x[col[p]];
      x[r] = acc * dinv[r];
    }
    __syncthreads();
  }
}

static inline unsigned grid_for(long long n, int tpb = 256) {
  long long g = (n + tpb - 1) / tpb;
  if (g < 1) g = 1;
  if (g > 152 * 16) g = 152 * 16;
  return (unsigned)g;
}

void launch_edge_rows(const c64* I, const c64* Phi, const c64* LpI, const c64* DZ,
                      const int32_t* n1, const int32_t* n2, double w, int m, c64* Y1, c64* U1,
                      cudaStream_t st) {
  if (m > 0) k_edge_rows<<<grid_for(m), 256, 0, st>>>(I, Phi, LpI, DZ, n1, n2, w, m, Y1, U1);
}
void launch_surf_rows(const c64* PQ, const c64* Phi, const int32_t* snode, const double* invP,
                      int ns, c64* Y2, c64* U2, cudaStream_t st) {
  if (ns > 0) k_surf_rows<<<grid_for(ns), 256, 0, st>>>(PQ, Phi, snode, invP, ns, Y2, U2);
}
void launch_node_rows(const c64* I, const c64* Q, const c64* Phi, const c64* U1, const c64* U2,
                      const int32_t* ne_ptr, const int32_t* ne_idx, const int32_t* ns_ptr,
                      const int32_t* ns_idx, const int32_t* yle_ptr, const int32_t* yle_col,
                      const c64* yle_val, double w, int n, c64* t, cudaStream_t st) {
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
void launch_trsv_level(const int32_t* rows, int nrows, const int32_t* ptr, const int32_t* col,
                       const c64* val, const c64* dinv, c64* x, cudaStream_t st) {
  k_trsv_level<<<grid_for(nrows), 256, 0, st>>>(rows, nrows, ptr, col, val, dinv, x);
}

}  // namespace peec

namespace peec {
void launch_trsv_tail(const int32_t* rows, const int32_t* lvl_off, int l0, int l1,
                      const int32_t* ptr, const int32_t* col, const c64* val, const c64* dinv,
                      c64* x, cudaStream_t st) {
  k_trsv_tail<<<1, 1024, 0, st>>>(rows, lvl_off, l0, l1, ptr, col, val, dinv, x);
}
}  // namespace peec
