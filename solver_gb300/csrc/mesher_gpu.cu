// Voxel mesher on the GPU: the same topology as the host mesher (mesher.cpp), built with
// per-cell kernels and prefix sums. The reference numbers voxels, nodes, edges and
// surfaces by its loop orders (create_volumes_mapping.jl, create_nodes_ref.jl,
// create_mapping_A{x,y,z}_v2.jl, create_A_mats_and_find_borders_with_map_Zs.jl,
// create_mapping_Gamma_no_rep.jl); here every numbered sequence is a flag per position of
// that loop order followed by an exclusive scan, so the numbers are the reference's.
//   occupancy   first grid holding each cell; voxel numbers by a scan in cell order
//   externals   per grid and cell the six external-face flags (create_Grids_externals.jl)
//   nodes       per grid in grid order (dominant grids first): the voxel's node on the 3N
//               lattice after the face resolution; dominant grids mark their offset nodes
//               in a flag array over the 3N lattice (the reference's sorted list), which the
//               other grids probe; the distinct nodes by a scan over the 3N lattice
//   edges       per lattice cell the first grid joining its two voxels with distinct
//               nodes; numbers by a scan in the family's loop order; incidence, material,
//               border and surface-impedance counters per edge
//   surfaces    twelve loop segments (three families, four each), a record per position
//               where the segment's first grid satisfies the face test; records by scans
// All outputs match mesher.cpp index for index (tests/test_gpu_mesher.py).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

// cudaSuccess and this file's success are both 0
#define MG_TRY(expr)                              \
  do {                                            \
    const int _e = (int)(expr);                   \
    if (_e != 0) return _e;                       \
  } while (0)

struct Geo {
  const uint8_t* g;  // G x N, x fastest
  int G, Nx, Ny, Nz;
  int64_t N;
  __device__ __forceinline__ bool at(int k, int x, int y, int z) const {
    return g[(int64_t)k * N + ((int64_t)z * Ny + y) * Nx + x] != 0;
  }
  __device__ __forceinline__ int64_t cell(int x, int y, int z) const {
    return ((int64_t)z * Ny + y) * Nx + x;
  }
};

// ------------------------------------------------------------------- exclusive scan
constexpr int SCAN_TPB = 256, SCAN_ITEMS = 4, SCAN_TILE = SCAN_TPB * SCAN_ITEMS;

__global__ void k_scan_tile(const int* __restrict__ in, int64_t n, int* out, int* sums) {
  __shared__ int ws[SCAN_TPB / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS], s = 0;
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    v[i] = base + i < n ? in[base + i] : 0;
    s += v[i];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = s;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < SCAN_TPB / 32 ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < SCAN_TPB / 32) ws[lane] = w;
  }
  __syncthreads();
  int run = incl - s + (wid > 0 ? ws[wid - 1] : 0);
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == SCAN_TPB - 1 && sums) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int* out, int64_t n, const int* __restrict__ offs) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / SCAN_TILE];
}

// out[i] = sum of in[0..i-1]; returns the total in *total (host)
int scan_exclusive(const int* in, int64_t n, int* out, int64_t* total, cudaStream_t st) {
  if (n <= 0) {
    *total = 0;
    return 0;
  }
  const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  int* sums = nullptr;
  MG_TRY(cudaMallocAsync(&sums, sizeof(int) * (nb + 1), st));
  k_scan_tile<<<(unsigned)nb, SCAN_TPB, 0, st>>>(in, n, out, sums);
  if (nb > 1) {
    int* offs = nullptr;
    MG_TRY(cudaMallocAsync(&offs, sizeof(int) * nb, st));
    int64_t dummy = 0;
    const int rc = scan_exclusive(sums, nb, offs, &dummy, st);
    if (rc) return rc;
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, offs);
    MG_TRY(cudaFreeAsync(offs, st));
  }
  int last_in = 0, last_out = 0;
  MG_TRY(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  MG_TRY(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  MG_TRY(cudaFreeAsync(sums, st));
  MG_TRY(cudaStreamSynchronize(st));
  *total = (int64_t)last_in + last_out;
  return 0;
}

// ------------------------------------------------------------------- occupancy, externals
__global__ void k_occupied(Geo M, int* flag) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < M.N;
       c += (int64_t)gridDim.x * blockDim.x) {
    int f = 0;
    for (int k = 0; k < M.G; ++k) f |= M.g[(int64_t)k * M.N + c];
    flag[c] = f != 0;
  }
}

// external-face flags of grid k at cell c, faces 0..5 = -y,+y,-x,+x,-z,+z
// (create_Grids_externals.jl: the boundary loops and the interior loop, ORed)
__global__ void k_externals(Geo M, uint8_t* E) {
  const int64_t total = (int64_t)M.G * M.N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / M.N);
    const int64_t c = i % M.N;
    const int x = (int)(c % M.Nx), y = (int)((c / M.Nx) % M.Ny), z = (int)(c / ((int64_t)M.Nx * M.Ny));
    uint8_t f[6] = {0, 0, 0, 0, 0, 0};
    if (M.at(k, x, y, z)) {
      const int n3[3] = {M.Nx, M.Ny, M.Nz};
      const int p[3] = {x, y, z};
      const int lo_face[3] = {2, 0, 4}, hi_face[3] = {3, 1, 5};
      for (int a = 0; a < 3; ++a) {
        const int n = n3[a], q = p[a];
        auto occ = [&](int d) {
          int qq[3] = {x, y, z};
          qq[a] = q + d;
          return M.at(k, qq[0], qq[1], qq[2]);
        };
        if (q == 0) {
          f[lo_face[a]] = 1;
          if (n > 1 && !occ(1)) f[hi_face[a]] = 1;
        }
        if (q == n - 1) {
          f[hi_face[a]] = 1;
          if (n > 1 && !occ(-1)) f[lo_face[a]] = 1;
        }
        if (q != 0 && q != n - 1) {
          if (!occ(-1)) f[lo_face[a]] = 1;
          if (!occ(1)) f[hi_face[a]] = 1;
        }
      }
    }
    for (int t = 0; t < 6; ++t) E[((int64_t)k * 6 + t) * M.N + c] = f[t];
  }
}

// ------------------------------------------------------------------- nodes
__device__ __forceinline__ int64_t node_id(int64_t c1, int64_t c2, int64_t c3, int Nx, int Ny) {
  return (c3 - 1) * (int64_t)(3 * Nx) * (3 * Ny) + (c2 - 1) * (int64_t)(3 * Nx) + c1;
}

__device__ __forceinline__ bool ext(const Geo& M, const uint8_t* E, int k, int f, int64_t c) {
  return E[((int64_t)k * 6 + f) * M.N + c] != 0;
}

// face flags and their resolution for one voxel of grid k (create_nodes_ref.jl:18-116)
__device__ bool face_offset(const Geo& M, const uint8_t* E, int k, int x, int y, int z, int& dx,
                            int& dy, int& dz) {
  const int64_t c = M.cell(x, y, z);
  bool f[6];
  for (int i = 0; i < 6; ++i) f[i] = ext(M, E, k, i, c);
  auto other = [&](int face, int xx, int yy, int zz) {
    const int64_t cc = M.cell(xx, yy, zz);
    for (int k2 = 0; k2 < M.G; ++k2)
      if (k2 != k && ext(M, E, k2, face, cc)) return true;
    return false;
  };
  bool fc[6] = {false, false, false, false, false, false};
  if (y > 1) fc[0] = other(1, x, y - 1, z);
  if (y + 2 <= M.Ny) fc[1] = other(0, x, y + 1, z);
  if (x > 1) fc[2] = other(3, x - 1, y, z);
  if (x + 2 <= M.Nx) fc[3] = other(2, x + 1, y, z);
  if (z > 1) fc[4] = other(5, x, y, z - 1);
  if (z + 2 <= M.Nz) fc[5] = other(4, x, y, z + 1);
  bool is[6];
  for (int a = 0; a < 3; ++a) {
    const int lo = 2 * a, hi = 2 * a + 1;
    is[lo] = f[lo];
    is[hi] = f[hi];
    if (f[lo] && f[hi]) {
      is[lo] = is[hi] = false;
      if (fc[lo] && !fc[hi]) is[lo] = true;
      else if (!fc[lo] && fc[hi]) is[hi] = true;
    }
  }
  dy = is[0] ? -1 : (is[1] ? 1 : 0);
  dx = is[2] ? -1 : (is[3] ? 1 : 0);
  dz = is[4] ? -1 : (is[5] ? 1 : 0);
  return is[0] || is[1] || is[2] || is[3] || is[4] || is[5];
}

// the voxels of grid k: dominant grids set their node and mark offset nodes in lista;
// the others take the first marked node among the 26 neighbours of the centre node
__constant__ int8_t c_probe[26][3] = {
    {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {1, -1, -1},
    {1, -1, 0},   {1, -1, 1},  {-1, 0, -1}, {-1, 0, 0},  {-1, 0, 1}, {0, 0, -1},  {0, 0, 1},
    {1, 0, -1},   {1, 0, 0},   {1, 0, 1},   {-1, 1, -1}, {-1, 1, 0}, {-1, 1, 1},  {0, 1, -1},
    {0, 1, 0},    {0, 1, 1},   {1, 1, -1},  {1, 1, 0},   {1, 1, 1}};

__global__ void k_nodes_grid(Geo M, const uint8_t* E, const int* vox_ex, int k, int dominant,
                             int64_t* nodes, int* lista) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < M.N;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(c % M.Nx), y = (int)((c / M.Nx) % M.Ny), z = (int)(c / ((int64_t)M.Nx * M.Ny));
    if (!M.at(k, x, y, z)) continue;
    const int64_t v = vox_ex[c];  // 0-based voxel number
    const int64_t c1 = 2 * (x + 1), c2 = 2 * (y + 1), c3 = 2 * (z + 1);
    int dx, dy, dz;
    if (face_offset(M, E, k, x, y, z, dx, dy, dz)) {
      if (dominant) {
        const int64_t id = node_id(c1 + dx, c2 + dy, c3 + dz, M.Nx, M.Ny);
        nodes[v] = id;
        lista[id] = 1;
      } else {
        int64_t found = -1;
        for (int p = 0; p < 26 && found < 0; ++p) {
          const int64_t cand =
              node_id(c1 + c_probe[p][0], c2 + c_probe[p][1], c3 + c_probe[p][2], M.Nx, M.Ny);
          if (lista[cand]) found = cand;
        }
        nodes[v] = found >= 0 ? found : node_id(c1 + dx, c2 + dy, c3 + dz, M.Nx, M.Ny);
      }
    } else {
      nodes[v] = node_id(c1, c2, c3, M.Nx, M.Ny);
    }
  }
}

__global__ void k_mark_nodes(const int64_t* nodes, int64_t nv, int* used) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x)
    used[nodes[v]] = 1;
}

__global__ void k_vox_node(const int64_t* nodes, int64_t nv, const int* rank, int64_t* vox_node) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv;
       v += (int64_t)gridDim.x * blockDim.x)
    vox_node[v] = rank[nodes[v]];
}

__global__ void k_compact_ids(const int* used, const int* rank, int64_t n, double* out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (used[i]) out[rank[i]] = (double)i;
}

__global__ void k_vox_map(const int* flag, const int* ex, int64_t N, int64_t* vox_map) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x)
    vox_map[c] = flag[c] ? ex[c] + 1 : 0;
}

// ------------------------------------------------------------------- edges
struct Edges {
  int64_t *n1, *n2, *cell, *mat, *b1, *b2, *zs;
};

__device__ __forceinline__ int64_t node_of(const Geo& M, const int* vox_ex, const int64_t* vox_node,
                                           int x, int y, int z) {
  return vox_node[vox_ex[M.cell(x, y, z)]];
}

// family d position t in its loop order (x: y, z, x; y: z, x, y; z: x, y, z, last fastest)
// -> the edge's first voxel and lattice cell
__device__ __forceinline__ void edge_pos(const Geo& M, int d, int64_t t, int& x, int& y, int& z,
                                         int64_t& lc) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  if (d == 0) {
    x = (int)(t % (Nx - 1));
    z = (int)((t / (Nx - 1)) % Nz);
    y = (int)(t / ((int64_t)(Nx - 1) * Nz));
    lc = ((int64_t)z * Ny + y) * (Nx - 1) + x;
  } else if (d == 1) {
    y = (int)(t % (Ny - 1));
    x = (int)((t / (Ny - 1)) % Nx);
    z = (int)(t / ((int64_t)(Ny - 1) * Nx));
    lc = ((int64_t)z * (Ny - 1) + y) * Nx + x;
  } else {
    z = (int)(t % (Nz - 1));
    y = (int)((t / (Nz - 1)) % Ny);
    x = (int)(t / ((int64_t)(Nz - 1) * Ny));
    lc = ((int64_t)z * Ny + y) * Nx + x;
  }
}

__device__ int edge_grid(const Geo& M, const int* vox_ex, const int64_t* vox_node, int d, int x,
                         int y, int z) {
  const int x2 = x + (d == 0), y2 = y + (d == 1), z2 = z + (d == 2);
  for (int k = 0; k < M.G; ++k)
    if (M.at(k, x, y, z) && M.at(k, x2, y2, z2)) {
      if (node_of(M, vox_ex, vox_node, x, y, z) != node_of(M, vox_ex, vox_node, x2, y2, z2))
        return k;
    }
  return -1;
}

__global__ void k_edge_flags(Geo M, const int* vox_ex, const int64_t* vox_node, int d, int64_t L,
                             int* flag, int* kk) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    int x, y, z;
    int64_t lc;
    edge_pos(M, d, t, x, y, z, lc);
    const int k = edge_grid(M, vox_ex, vox_node, d, x, y, z);
    flag[t] = k >= 0;
    kk[t] = k;
  }
}

// incidence, material, borders and surface-impedance counters
// (create_A_mats_and_find_borders_with_map_Zs.jl, as mesher.cpp restates it)
__global__ void k_edge_fill(Geo M, const int* vox_ex, const int64_t* vox_node, int d, int64_t L,
                            const int* flag, const int* kk, const int* num, int64_t base,
                            const double* sigma, Edges E) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[t]) continue;
    int x, y, z;
    int64_t lc;
    edge_pos(M, d, t, x, y, z, lc);
    const int k = kk[t];
    const int64_t e = base + num[t];
    const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
    auto G = [&](int xx, int yy, int zz) { return M.at(k, xx, yy, zz); };
    E.n1[e] = node_of(M, vox_ex, vox_node, x, y, z);
    E.n2[e] = node_of(M, vox_ex, vox_node, x + (d == 0), y + (d == 1), z + (d == 2));
    E.cell[e] = lc;
    E.mat[e] = k + 1;
    int64_t zs[4] = {0, 0, 0, 0};
    int64_t b1 = 0, b2 = 0;
    if (d == 0) {
      if (sigma[k] != 0) {
        if (z == 0 || z == Nz - 1) { zs[0] += 1; zs[1] += 1; }
        else {
          if (!G(x, y, z - 1)) zs[0] += 1;
          if (!G(x + 1, y, z - 1)) zs[1] += 1;
          if (!G(x, y, z + 1)) zs[0] += 1;
          if (!G(x + 1, y, z + 1)) zs[1] += 1;
        }
        if (y == 0 || y == Ny - 1) { zs[2] += 1; zs[3] += 1; }
        else {
          if (!G(x, y - 1, z)) zs[2] += 1;
          if (!G(x + 1, y - 1, z)) zs[3] += 1;
          if (!G(x, y + 1, z)) zs[2] += 1;
          if (!G(x + 1, y + 1, z)) zs[3] += 1;
        }
      }
      if (x > 0) { if (!G(x - 1, y, z)) b1 = k + 1; }
      else b1 = k + 1;
      if (x + 2 == Nx) b2 = k + 1;
      else if (x + 2 <= Nx - 1 && !G(x + 2, y, z)) b2 = k + 1;
    } else if (d == 1) {
      if (sigma[k] != 0) {
        if (z == 0 || z == Nz - 1) { zs[0] += 1; zs[1] += 1; }
        else {
          if (!G(x, y, z - 1)) zs[0] += 1;
          if (!G(x, y + 1, z - 1)) zs[1] += 1;
          if (!G(x, y, z + 1)) zs[0] += 1;
          if (!G(x, y + 1, z + 1)) zs[1] += 1;
        }
        if (x == 0 || x == Nx - 1) { zs[2] += 1; zs[3] += 1; }
        else {
          if (!G(x - 1, y, z)) zs[2] += 1;
          if (!G(x - 1, y + 1, z)) zs[3] += 1;
          if (!G(x + 1, y, z)) zs[2] += 1;
          if (!G(x + 1, y + 1, z)) zs[3] += 1;
        }
      }
      if (y > 0) { if (!G(x, y - 1, z)) b1 = k + 1; }
      else b1 = k + 1;
      if (y + 2 == Ny) b2 = k + 1;
      else if (y + 2 <= Ny - 1 && !G(x, y + 2, z)) b2 = k + 1;
    } else {
      if (sigma[k] != 0) {
        // the +1 side tests the z-level of the first voxel for both counters, as the
        // reference does
        if (x == 0 || x == Nx - 1) { zs[0] += 1; zs[1] += 1; }
        else {
          if (!G(x - 1, y, z)) zs[0] += 1;
          if (!G(x - 1, y, z + 1)) zs[1] += 1;
          if (!G(x + 1, y, z)) zs[0] += 1;
          if (!G(x + 1, y, z)) zs[1] += 1;
        }
        if (y == 0 || y == Ny - 1) { zs[2] += 1; zs[3] += 1; }
        else {
          if (!G(x, y - 1, z)) zs[2] += 1;
          if (!G(x, y - 1, z + 1)) zs[3] += 1;
          if (!G(x, y + 1, z)) zs[2] += 1;
          if (!G(x, y + 1, z)) zs[3] += 1;
        }
      }
      if (z > 0) { if (!G(x, y, z - 1)) b1 = k + 1; }
      else b1 = k + 1;
      if (z + 2 == Nz) b2 = k + 1;
      else if (z + 2 <= Nz - 1 && !G(x, y, z + 2)) b2 = k + 1;
    }
    for (int i = 0; i < 4; ++i) E.zs[4 * e + i] = zs[i];
    E.b1[e] = b1;
    E.b2[e] = b2;
  }
}

// ------------------------------------------------------------------- surfaces
// segment s (0..11) of create_mapping_Gamma_no_rep.jl as mesher.cpp orders them: per family
// (0: y-normal, 1: x-normal, 2: z-normal) lower boundary, lower interior, upper boundary,
// upper interior. Length of a segment's loop:
__host__ __device__ inline int64_t seg_len(int s, int Nx, int Ny, int Nz) {
  switch (s) {
    case 0: case 2: return (int64_t)Nx * Nz;
    case 1: case 3: return (int64_t)Nx * (Ny - 1) * Nz;
    case 4: case 6: return (int64_t)Ny * Nz;
    case 5: case 7: return (int64_t)(Nx - 1) * Ny * Nz;
    case 8: case 10: return (int64_t)Nx * Ny;
    default: return (int64_t)Nx * Ny * (Nz - 1);
  }
}

// whether position t of segment s records a surface, and its lattice cell and voxel
__device__ bool seg_eval(const Geo& M, const uint8_t* E, int s, int64_t t, int64_t& lat, int& vx,
                         int& vy, int& vz) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  auto G = [&](int k, int x, int y, int z) { return M.at(k, x, y, z); };
  auto any_other = [&](int k, bool ok, int x, int y, int z) {
    if (!ok) return false;
    for (int k2 = 0; k2 < M.G; ++k2)
      if (k2 != k && G(k2, x, y, z)) return true;
    return false;
  };
  auto c12 = [&](int x, int yf, int z) { return ((int64_t)z * (Ny + 1) + yf) * Nx + x; };
  auto c34 = [&](int xf, int y, int z) { return ((int64_t)z * Ny + y) * (Nx + 1) + xf; };
  auto c56 = [&](int x, int y, int zf) { return ((int64_t)zf * Ny + y) * Nx + x; };
  int x = 0, y = 0, z = 0;
  switch (s) {
    case 0: x = (int)(t / Nz); z = (int)(t % Nz); y = 0; break;
    case 1: z = (int)(t % Nz); y = 1 + (int)((t / Nz) % (Ny - 1)); x = (int)(t / ((int64_t)Nz * (Ny - 1))); break;
    case 2: x = (int)(t / Nz); z = (int)(t % Nz); y = Ny - 1; break;
    case 3: z = (int)(t % Nz); y = (int)((t / Nz) % (Ny - 1)); x = (int)(t / ((int64_t)Nz * (Ny - 1))); break;
    case 4: y = (int)(t / Nz); z = (int)(t % Nz); x = 0; break;
    case 5: z = (int)(t % Nz); y = (int)((t / Nz) % Ny); x = 1 + (int)(t / ((int64_t)Nz * Ny)); break;
    case 6: y = (int)(t / Nz); z = (int)(t % Nz); x = Nx - 1; break;
    case 7: z = (int)(t % Nz); y = (int)((t / Nz) % Ny); x = (int)(t / ((int64_t)Nz * Ny)); break;
    case 8: x = (int)(t / Ny); y = (int)(t % Ny); z = 0; break;
    case 9: z = 1 + (int)(t % (Nz - 1)); y = (int)((t / (Nz - 1)) % Ny); x = (int)(t / ((int64_t)(Nz - 1) * Ny)); break;
    case 10: x = (int)(t / Ny); y = (int)(t % Ny); z = Nz - 1; break;
    default: z = (int)(t % (Nz - 1)); y = (int)((t / (Nz - 1)) % Ny); x = (int)(t / ((int64_t)(Nz - 1) * Ny)); break;
  }
  vx = x; vy = y; vz = z;
  const int64_t c = M.cell(x, y, z);
  for (int k = 0; k < M.G; ++k) {
    switch (s) {
      case 0: {
        const bool om = any_other(k, y + 1 <= Ny - 1, x, y + 1, z);
        if (G(k, x, y, z) && (!ext(M, E, k, 1, c) || om)) { lat = c12(x, y, z); return true; }
        break;
      }
      case 1: {
        const bool om = any_other(k, y + 1 <= Ny - 1, x, y + 1, z);
        if (G(k, x, y, z) && !G(k, x, y - 1, z) && (!ext(M, E, k, 1, c) || om)) {
          lat = c12(x, y, z);
          return true;
        }
        break;
      }
      case 2: {
        const bool om = any_other(k, y - 1 >= 0, x, y - 1, z);
        if (G(k, x, y, z) && (!ext(M, E, k, 0, c) || om)) { lat = c12(x, y + 1, z); return true; }
        break;
      }
      case 3: {
        const bool om = any_other(k, y - 1 >= 0, x, y - 1, z);
        if (G(k, x, y, z) && !G(k, x, y + 1, z) && (!ext(M, E, k, 0, c) || om)) {
          if (any_other(k, true, x, y + 1, z)) return false;
          lat = c12(x, y + 1, z);
          return true;
        }
        break;
      }
      case 4: {
        const bool om = any_other(k, x + 1 <= Nx - 1, x + 1, y, z);
        if (G(k, x, y, z) && (!ext(M, E, k, 3, c) || om)) { lat = c34(x, y, z); return true; }
        break;
      }
      case 5: {
        const bool om = any_other(k, x + 1 <= Nx - 1, x + 1, y, z);
        if (G(k, x, y, z) && !G(k, x - 1, y, z) && (!ext(M, E, k, 3, c) || om)) {
          lat = c34(x, y, z);
          return true;
        }
        break;
      }
      case 6: {
        const bool om = any_other(k, x - 1 >= 0, x - 1, y, z);
        if (G(k, x, y, z) && (!ext(M, E, k, 2, c) || om)) { lat = c34(x + 1, y, z); return true; }
        break;
      }
      case 7: {
        const bool om = any_other(k, x - 1 >= 0, x - 1, y, z);
        if (G(k, x, y, z) && !G(k, x + 1, y, z) && (!ext(M, E, k, 2, c) || om)) {
          if (any_other(k, true, x + 1, y, z)) return false;
          lat = c34(x + 1, y, z);
          return true;
        }
        break;
      }
      case 8: {
        const bool om = any_other(k, z + 1 <= Nz - 1, x, y, z + 1);
        if (G(k, x, y, z) && (!ext(M, E, k, 5, c) || om)) { lat = c56(x, y, z); return true; }
        break;
      }
      case 9: {
        const bool om = any_other(k, z + 1 <= Nz - 1, x, y, z + 1);
        if (G(k, x, y, z) && !G(k, x, y, z - 1) && (!ext(M, E, k, 5, c) || om)) {
          lat = c56(x, y, z);
          return true;
        }
        break;
      }
      case 10: {
        const bool om = any_other(k, z - 1 >= 0, x, y, z - 1);
        if (G(k, x, y, z) && (!ext(M, E, k, 4, c) || om)) { lat = c56(x, y, z + 1); return true; }
        break;
      }
      default: {
        const bool om = any_other(k, z - 1 >= 0, x, y, z - 1);
        if (G(k, x, y, z) && !G(k, x, y, z + 1) && (!ext(M, E, k, 4, c) || om)) {
          if (any_other(k, true, x, y, z + 1)) return false;
          lat = c56(x, y, z + 1);
          return true;
        }
        break;
      }
    }
  }
  return false;
}

__global__ void k_seg_flags(Geo M, const uint8_t* E, int s, int64_t L, int* flag) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t lat;
    int x, y, z;
    flag[t] = seg_eval(M, E, s, t, lat, x, y, z);
  }
}

__global__ void k_seg_fill(Geo M, const uint8_t* E, const int* vox_ex, const int64_t* vox_node,
                           int s, int64_t L, const int* flag, const int* num, int64_t base,
                           int64_t* snode, int64_t* sfam, int64_t* scell) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < L;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (!flag[t]) continue;
    int64_t lat;
    int x, y, z;
    seg_eval(M, E, s, t, lat, x, y, z);
    const int64_t r = base + num[t];
    snode[r] = node_of(M, vox_ex, vox_node, x, y, z);
    sfam[r] = s / 4;
    scell[r] = lat;
  }
}

struct MeshOut {
  std::map<std::string, std::vector<int64_t>> iarr;
  std::map<std::string, std::vector<double>> darr;
  std::string err;
};

template <typename T>
int to_host(std::vector<T>& h, const T* d, int64_t n) {
  h.resize((size_t)n);
  if (n > 0) MG_TRY(cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost));
  return 0;
}

unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

// frees what it allocated on every path
struct DevPool {
  std::vector<void*> p;
  template <typename T>
  int alloc(T** out, int64_t n) {
    *out = nullptr;
    const size_t bytes = sizeof(T) * (size_t)(n > 0 ? n : 1);
    MG_TRY(cudaMalloc((void**)out, bytes));
    p.push_back(*out);
    return 0;
  }
  ~DevPool() {
    for (void* q : p) cudaFree(q);
  }
};

int mesh_gpu(MeshOut& O, const uint8_t* grids, int G, int Nx, int Ny, int Nz,
             const uint8_t* dominant, const double* sigma) {
  cudaStream_t st = nullptr;
  MG_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{st};
  DevPool P;
  const int64_t N = (int64_t)Nx * Ny * Nz;
  uint8_t* dg;
  MG_TRY(P.alloc(&dg, (int64_t)G * N));
  MG_TRY(cudaMemcpyAsync(dg, grids, (size_t)G * N, cudaMemcpyHostToDevice, st));
  double* dsig;
  MG_TRY(P.alloc(&dsig, G));
  MG_TRY(cudaMemcpyAsync(dsig, sigma, sizeof(double) * G, cudaMemcpyHostToDevice, st));
  Geo M{dg, G, Nx, Ny, Nz, N};
  // voxels
  int *occ, *vox_ex;
  int64_t* vox_map;
  MG_TRY(P.alloc(&occ, N));
  MG_TRY(P.alloc(&vox_ex, N));
  MG_TRY(P.alloc(&vox_map, N));
  k_occupied<<<blocks_for(N), 256, 0, st>>>(M, occ);
  int64_t nv = 0;
  MG_TRY(scan_exclusive(occ, N, vox_ex, &nv, st));
  k_vox_map<<<blocks_for(N), 256, 0, st>>>(occ, vox_ex, N, vox_map);
  // externals
  uint8_t* E;
  MG_TRY(P.alloc(&E, (int64_t)G * 6 * N));
  k_externals<<<blocks_for((int64_t)G * N), 256, 0, st>>>(M, E);
  // nodes on the 3N lattice (ids 1 .. 27 N)
  const int64_t NF = (int64_t)27 * N + 1;
  int64_t* nodes;
  int *lista, *used, *rank;
  MG_TRY(P.alloc(&nodes, nv));
  MG_TRY(P.alloc(&lista, NF));
  MG_TRY(P.alloc(&used, NF));
  MG_TRY(P.alloc(&rank, NF));
  MG_TRY(cudaMemsetAsync(lista, 0, sizeof(int) * NF, st));
  MG_TRY(cudaMemsetAsync(used, 0, sizeof(int) * NF, st));
  for (int pass = 0; pass < 2; ++pass)
    for (int k = 0; k < G; ++k) {
      const int dom = dominant[k] != 0;
      if (dom != (pass == 0)) continue;
      k_nodes_grid<<<blocks_for(N), 256, 0, st>>>(M, E, vox_ex, k, dom, nodes, lista);
    }
  k_mark_nodes<<<blocks_for(nv), 256, 0, st>>>(nodes, nv, used);
  int64_t nn = 0;
  MG_TRY(scan_exclusive(used, NF, rank, &nn, st));
  int64_t* vox_node;
  double* nodes_red;
  MG_TRY(P.alloc(&vox_node, nv));
  MG_TRY(P.alloc(&nodes_red, nn));
  k_vox_node<<<blocks_for(nv), 256, 0, st>>>(nodes, nv, rank, vox_node);
  k_compact_ids<<<blocks_for(NF), 256, 0, st>>>(used, rank, NF, nodes_red);
  // edges, family by family in the reference's loop order
  const int64_t Lf[3] = {(int64_t)(Nx > 1 ? Nx - 1 : 0) * Ny * Nz,
                         (int64_t)Nx * (Ny > 1 ? Ny - 1 : 0) * Nz,
                         (int64_t)Nx * Ny * (Nz > 1 ? Nz - 1 : 0)};
  const int64_t Lmax = std::max(Lf[0], std::max(Lf[1], Lf[2]));
  int *ef, *ek, *en;
  MG_TRY(P.alloc(&ef, Lmax));
  MG_TRY(P.alloc(&ek, Lmax));
  MG_TRY(P.alloc(&en, Lmax));
  int64_t mcount[3] = {0, 0, 0};
  std::vector<std::vector<int>> fl(3), kk(3), nm(3);
  // count first (numbers need the totals of the earlier families for the offsets)
  int* fstore[3];
  int* kstore[3];
  int* nstore[3];
  for (int d = 0; d < 3; ++d) {
    MG_TRY(P.alloc(&fstore[d], Lf[d]));
    MG_TRY(P.alloc(&kstore[d], Lf[d]));
    MG_TRY(P.alloc(&nstore[d], Lf[d]));
    if (Lf[d] == 0) continue;
    k_edge_flags<<<blocks_for(Lf[d]), 256, 0, st>>>(M, vox_ex, vox_node, d, Lf[d], fstore[d],
                                                   kstore[d]);
    MG_TRY(scan_exclusive(fstore[d], Lf[d], nstore[d], &mcount[d], st));
  }
  const int64_t m = mcount[0] + mcount[1] + mcount[2];
  Edges ED;
  MG_TRY(P.alloc(&ED.n1, m));
  MG_TRY(P.alloc(&ED.n2, m));
  MG_TRY(P.alloc(&ED.cell, m));
  MG_TRY(P.alloc(&ED.mat, m));
  MG_TRY(P.alloc(&ED.b1, m));
  MG_TRY(P.alloc(&ED.b2, m));
  MG_TRY(P.alloc(&ED.zs, 4 * m));
  int64_t ebase = 0;
  for (int d = 0; d < 3; ++d) {
    if (Lf[d] > 0)
      k_edge_fill<<<blocks_for(Lf[d]), 256, 0, st>>>(M, vox_ex, vox_node, d, Lf[d], fstore[d],
                                                    kstore[d], nstore[d], ebase, dsig, ED);
    ebase += mcount[d];
  }
  // surfaces, twelve segments
  int64_t scount[12];
  int* sf[12];
  int* sn[12];
  for (int s = 0; s < 12; ++s) {
    const int64_t L = std::max<int64_t>(seg_len(s, Nx, Ny, Nz), 0);
    MG_TRY(P.alloc(&sf[s], L));
    MG_TRY(P.alloc(&sn[s], L));
    scount[s] = 0;
    if (L == 0) continue;
    k_seg_flags<<<blocks_for(L), 256, 0, st>>>(M, E, s, L, sf[s]);
    MG_TRY(scan_exclusive(sf[s], L, sn[s], &scount[s], st));
  }
  int64_t ns = 0, nsf[3] = {0, 0, 0};
  for (int s = 0; s < 12; ++s) {
    ns += scount[s];
    nsf[s / 4] += scount[s];
  }
  int64_t *snode, *sfam, *scell;
  MG_TRY(P.alloc(&snode, ns));
  MG_TRY(P.alloc(&sfam, ns));
  MG_TRY(P.alloc(&scell, ns));
  int64_t sbase = 0;
  for (int s = 0; s < 12; ++s) {
    const int64_t L = std::max<int64_t>(seg_len(s, Nx, Ny, Nz), 0);
    if (L > 0)
      k_seg_fill<<<blocks_for(L), 256, 0, st>>>(M, E, vox_ex, vox_node, s, L, sf[s], sn[s],
                                               sbase, snode, sfam, scell);
    sbase += scount[s];
  }
  MG_TRY(cudaGetLastError());
  MG_TRY(cudaStreamSynchronize(st));
  // host copies, named as the host mesher names them
  auto& I = O.iarr;
  MG_TRY(to_host(I["vox_map"], vox_map, N));
  MG_TRY(to_host(I["vox_node"], vox_node, nv));
  I["counts"] = {nv, nn, mcount[0], mcount[1], mcount[2], nsf[0], nsf[1], nsf[2]};
  MG_TRY(to_host(I["edge_n1"], ED.n1, m));
  MG_TRY(to_host(I["edge_n2"], ED.n2, m));
  MG_TRY(to_host(I["edge_cell"], ED.cell, m));
  MG_TRY(to_host(I["edge_mat"], ED.mat, m));
  MG_TRY(to_host(I["edge_border1"], ED.b1, m));
  MG_TRY(to_host(I["edge_border2"], ED.b2, m));
  MG_TRY(to_host(I["edge_zs"], ED.zs, 4 * m));
  MG_TRY(to_host(I["surf_node"], snode, ns));
  MG_TRY(to_host(I["surf_fam"], sfam, ns));
  MG_TRY(to_host(I["surf_cell"], scell, ns));
  std::vector<int64_t> hn;
  MG_TRY(to_host(hn, nodes, nv));
  O.darr["nodes"].assign(hn.begin(), hn.end());
  MG_TRY(to_host(O.darr["nodes_red"], nodes_red, nn));
  return 0;
}

}  // namespace

extern "C" {

// The GPU form of peec_mesh_build (mesher.cpp): grids is G x Nx x Ny x Nz uint8, x fastest
// per grid; dominant[k] != 0 marks conductor grids; sigma[k] the conductivity. Runs on
// device `device` (the caller's current device is restored). Returns a handle read with
// peec_mesh_gpu_len / peec_mesh_gpu_copy, or NULL (the message in *err_out, if given,
// until the next call on this thread).
void* peec_mesh_gpu_build(const uint8_t* grids, int G, int Nx, int Ny, int Nz,
                          const uint8_t* dominant, const double* sigma, int device,
                          const char** err_out) {
  static thread_local std::string last;
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) {
    last = "peec_mesh_gpu_build: cannot select the device";
    if (err_out) *err_out = last.c_str();
    return nullptr;
  }
  struct Restore {
    int d;
    ~Restore() { if (d >= 0) cudaSetDevice(d); }
  } restore{prev};
  if (G <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || !grids || !dominant || !sigma) {
    last = "peec_mesh_gpu_build: bad arguments";
    if (err_out) *err_out = last.c_str();
    return nullptr;
  }
  if ((int64_t)27 * Nx * Ny * Nz + 1 > INT32_MAX) {
    last = "peec_mesh_gpu_build: grid too large (27 Nx Ny Nz must fit in int32)";
    if (err_out) *err_out = last.c_str();
    return nullptr;
  }
  MeshOut* O = new MeshOut();
  const int rc = mesh_gpu(*O, grids, G, Nx, Ny, Nz, dominant, sigma);
  if (rc) {
    last = std::string("peec_mesh_gpu_build: CUDA error ") + cudaGetErrorString((cudaError_t)rc);
    if (err_out) *err_out = last.c_str();
    delete O;
    return nullptr;
  }
  return O;
}

int64_t peec_mesh_gpu_len(void* h, const char* name, int* is_double) {
  MeshOut* O = static_cast<MeshOut*>(h);
  auto it = O->iarr.find(name);
  if (it != O->iarr.end()) { if (is_double) *is_double = 0; return (int64_t)it->second.size(); }
  auto jt = O->darr.find(name);
  if (jt != O->darr.end()) { if (is_double) *is_double = 1; return (int64_t)jt->second.size(); }
  return -1;
}

int peec_mesh_gpu_copy(void* h, const char* name, void* out) {
  MeshOut* O = static_cast<MeshOut*>(h);
  auto it = O->iarr.find(name);
  if (it != O->iarr.end()) {
    if (!it->second.empty()) memcpy(out, it->second.data(), it->second.size() * sizeof(int64_t));
    return 0;
  }
  auto jt = O->darr.find(name);
  if (jt != O->darr.end()) {
    if (!jt->second.empty()) memcpy(out, jt->second.data(), jt->second.size() * sizeof(double));
    return 0;
  }
  return -1;
}

void peec_mesh_gpu_free(void* h) { delete static_cast<MeshOut*>(h); }

}  // extern "C"
