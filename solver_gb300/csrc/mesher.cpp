// Voxel mesher for the FFT-PEEC solver: turns per-material boolean voxel grids
// into the topology the circulant operator consumes (nodes, inductive edges,
// charge surfaces, lattice placement of both, border/surface-impedance flags).
//
// This is host setup, run once per geometry. It follows the reference mesher
// step for step because every downstream index (edge order, surface order,
// node order) must agree with it:
//   src/lib/solverFFT/create_volumes_mapping.jl:1-23      voxel numbering
//   src/lib/solverFFT/create_Grids_externals.jl:1-261     external-face flags
//   src/lib/solverFFT/create_nodes_ref.jl:1-432           node placement/merging
//   src/lib/solverFFT/create_mapping_A{x,y,z}_v2.jl:1-29  edge numbering
//   src/lib/solverFFT/create_A_mats_and_find_borders_with_map_Zs.jl:1-229
//   src/lib/solverFFT/create_mapping_Gamma_no_rep.jl:1-421 surfaces + Gamma
// Loop orders below are the reference's loop orders: they fix the numbering. Loops run
// in parallel (OpenMP) where that cannot change the result: per-cell predicates are
// evaluated in parallel, and every numbered sequence is assembled from per-slab pieces
// concatenated in the reference's slab order, so the output is the same for any number
// of threads.
// All indices here are 0-based; the Python wrapper converts where needed.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct Mesh {
  int G = 0, Nx = 0, Ny = 0, Nz = 0;
  std::vector<uint8_t> g;         // G * Nx*Ny*Nz, x fastest
  std::vector<int64_t> vox_map;   // cell -> voxel number (1-based), 0 = empty
  int64_t num_vox = 0;
  std::vector<double> nodes;      // per voxel number-1: node id on the 3N lattice
  std::vector<double> nodes_red;  // sorted unique node ids
  std::vector<int64_t> vox_node;  // per voxel number-1: 0-based node index
  // edges, family d = 0,1,2 (x,y,z); stored already in edge-number order
  int64_t m[3] = {0, 0, 0};
  std::vector<int64_t> e_n1[3], e_n2[3], e_cell[3], e_mat[3];
  std::vector<int64_t> e_border1[3], e_border2[3];
  std::vector<int64_t> e_zs[3];   // 4 counters per edge (maps_Zs kind a: [1],[2]; kind b: [1],[2])
  // surfaces in surface-number order
  int64_t ns_fam[3] = {0, 0, 0};
  std::vector<int64_t> s_node, s_fam, s_cell;
  std::map<std::string, std::vector<int64_t>> iarr;
  std::map<std::string, std::vector<double>> darr;

  inline bool at(int k, int x, int y, int z) const {
    return g[(size_t)k * Nx * Ny * Nz + ((size_t)z * Ny + y) * Nx + x] != 0;
  }
  inline size_t cell(int x, int y, int z) const { return ((size_t)z * Ny + y) * Nx + x; }
};

// ext[k][f][cell], f = 0..5 for reference faces 1..6 (-y,+y,-x,+x,-z,+z)
struct Ext {
  int G, N;
  std::vector<uint8_t> v;
  Ext(int G_, int N_) : G(G_), N(N_), v((size_t)G_ * 6 * N_, 0) {}
  inline uint8_t& operator()(int k, int f, size_t c) { return v[((size_t)k * 6 + f) * N + c]; }
  inline uint8_t get(int k, int f, size_t c) const { return v[((size_t)k * 6 + f) * N + c]; }
};

void build_externals(const Mesh& M, Ext& E) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  // x boundaries (create_Grids_externals.jl:15-37)
  for (int z = 0; z < Nz; ++z)
    for (int y = 0; y < Ny; ++y)
      for (int k = 0; k < M.G; ++k) {
        if (M.at(k, 0, y, z)) {
          E(k, 2, M.cell(0, y, z)) = 1;
          if (Nx > 1 && !M.at(k, 1, y, z)) E(k, 3, M.cell(0, y, z)) = 1;
        }
        int x = Nx - 1;
        if (M.at(k, x, y, z)) {
          E(k, 3, M.cell(x, y, z)) = 1;
          if (Nx > 1 && !M.at(k, x - 1, y, z)) E(k, 2, M.cell(x, y, z)) = 1;
        }
      }
  // y boundaries (:70-91)
  for (int z = 0; z < Nz; ++z)
    for (int x = 0; x < Nx; ++x)
      for (int k = 0; k < M.G; ++k) {
        if (M.at(k, x, 0, z)) {
          E(k, 0, M.cell(x, 0, z)) = 1;
          if (Ny > 1 && !M.at(k, x, 1, z)) E(k, 1, M.cell(x, 0, z)) = 1;
        }
        int y = Ny - 1;
        if (M.at(k, x, y, z)) {
          E(k, 1, M.cell(x, y, z)) = 1;
          if (Ny > 1 && !M.at(k, x, y - 1, z)) E(k, 0, M.cell(x, y, z)) = 1;
        }
      }
  // z boundaries
  for (int y = 0; y < Ny; ++y)
    for (int x = 0; x < Nx; ++x)
      for (int k = 0; k < M.G; ++k) {
        if (M.at(k, x, y, 0)) {
          E(k, 4, M.cell(x, y, 0)) = 1;
          if (Nz > 1 && !M.at(k, x, y, 1)) E(k, 5, M.cell(x, y, 0)) = 1;
        }
        int z = Nz - 1;
        if (M.at(k, x, y, z)) {
          E(k, 5, M.cell(x, y, z)) = 1;
          if (Nz > 1 && !M.at(k, x, y, z - 1)) E(k, 4, M.cell(x, y, z)) = 1;
        }
      }
  // interior faces (each cell's flags are written by its own iteration)
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; ++z)
    for (int y = 0; y < Ny; ++y)
      for (int x = 0; x < Nx; ++x)
        for (int k = 0; k < M.G; ++k) {
          if (!M.at(k, x, y, z)) continue;
          size_t c = M.cell(x, y, z);
          if (x != 0 && x != Nx - 1) {
            if (!M.at(k, x - 1, y, z)) E(k, 2, c) = 1;
            if (!M.at(k, x + 1, y, z)) E(k, 3, c) = 1;
          }
          if (y != 0 && y != Ny - 1) {
            if (!M.at(k, x, y - 1, z)) E(k, 0, c) = 1;
            if (!M.at(k, x, y + 1, z)) E(k, 1, c) = 1;
          }
          if (z != 0 && z != Nz - 1) {
            if (!M.at(k, x, y, z - 1)) E(k, 4, c) = 1;
            if (!M.at(k, x, y, z + 1)) E(k, 5, c) = 1;
          }
        }
}

inline double node_id(int64_t c1, int64_t c2, int64_t c3, int Nx, int Ny) {
  // from_3D_to_1D(c1, c2, c3, 3Nx, 3Ny) with 1-based fine-lattice coordinates
  return (double)((c3 - 1) * (int64_t)(3 * Nx) * (3 * Ny) + (c2 - 1) * (int64_t)(3 * Nx) + c1);
}

// Face flags and their resolution for one voxel of grid k
// (create_nodes_ref.jl:18-116). Returns the node offset (dx,dy,dz) and whether
// any external face survived the resolution.
bool face_offset(const Mesh& M, const Ext& E, int k, int x, int y, int z, int& dx, int& dy,
                 int& dz) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  size_t c = M.cell(x, y, z);
  bool f[6];
  for (int i = 0; i < 6; ++i) f[i] = E.get(k, i, c);
  bool fc[6] = {false, false, false, false, false, false};
  // the "- 1 > 1" tests are strict in the reference (1-based index > 2)
  auto other = [&](int face, int xx, int yy, int zz) {
    for (int k2 = 0; k2 < M.G; ++k2)
      if (k2 != k && E.get(k2, face, M.cell(xx, yy, zz))) return true;
    return false;
  };
  if (y + 1 - 1 > 1) fc[0] = other(1, x, y - 1, z);
  if (y + 1 + 1 <= Ny) fc[1] = other(0, x, y + 1, z);
  if (x + 1 - 1 > 1) fc[2] = other(3, x - 1, y, z);
  if (x + 1 + 1 <= Nx) fc[3] = other(2, x + 1, y, z);
  if (z + 1 - 1 > 1) fc[4] = other(5, x, y, z - 1);
  if (z + 1 + 1 <= Nz) fc[5] = other(4, x, y, z + 1);
  bool is[6];
  for (int a = 0; a < 3; ++a) {
    int lo = 2 * a, hi = 2 * a + 1;
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

void build_nodes(Mesh& M, const Ext& E, const std::vector<uint8_t>& dominant) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  M.nodes.assign(M.num_vox, 0.0);
  std::vector<double> lista;
  // dominant (conductor) grids first, in grid order (create_nodes_ref.jl:9-226). Within a
  // grid every voxel is set once and lista is sorted afterwards, so the cells can be
  // visited in any order: plane by plane, in parallel.
  for (int k = 0; k < M.G; ++k) {
    if (!dominant[k]) continue;
#pragma omp parallel
    {
      std::vector<double> loc;
#pragma omp for schedule(static)
      for (int z = 0; z < Nz; ++z)
        for (int y = 0; y < Ny; ++y)
          for (int x = 0; x < Nx; ++x) {
            if (!M.at(k, x, y, z)) continue;
            int64_t c1 = 2 * (x + 1), c2 = 2 * (y + 1), c3 = 2 * (z + 1);
            int dx, dy, dz;
            size_t v = M.vox_map[M.cell(x, y, z)] - 1;
            if (face_offset(M, E, k, x, y, z, dx, dy, dz)) {
              M.nodes[v] = node_id(c1 + dx, c2 + dy, c3 + dz, Nx, Ny);
              loc.push_back(M.nodes[v]);
            } else {
              M.nodes[v] = node_id(c1, c2, c3, Nx, Ny);
            }
          }
#pragma omp critical
      lista.insert(lista.end(), loc.begin(), loc.end());
    }
  }
  std::sort(lista.begin(), lista.end());
  lista.erase(std::unique(lista.begin(), lista.end()), lista.end());
  // non-dominant grids reuse a neighbouring dominant node when one exists
  // (create_nodes_ref.jl:227-425, build_nodes :440-488 gives the probe order)
  static const int probe[26][3] = {
      {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {0, -1, -1}, {0, -1, 0}, {0, -1, 1}, {1, -1, -1},
      {1, -1, 0},   {1, -1, 1},  {-1, 0, -1}, {-1, 0, 0},  {-1, 0, 1}, {0, 0, -1},  {0, 0, 1},
      {1, 0, -1},   {1, 0, 0},   {1, 0, 1},   {-1, 1, -1}, {-1, 1, 0}, {-1, 1, 1},  {0, 1, -1},
      {0, 1, 0},    {0, 1, 1},   {1, 1, -1},  {1, 1, 0},   {1, 1, 1}};
  for (int k = 0; k < M.G; ++k) {
    if (dominant[k]) continue;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < Nz; ++z)
      for (int y = 0; y < Ny; ++y)
        for (int x = 0; x < Nx; ++x) {
          if (!M.at(k, x, y, z)) continue;
          int64_t c1 = 2 * (x + 1), c2 = 2 * (y + 1), c3 = 2 * (z + 1);
          int dx, dy, dz;
          size_t v = M.vox_map[M.cell(x, y, z)] - 1;
          if (face_offset(M, E, k, x, y, z, dx, dy, dz)) {
            double found = 0.0;
            bool hit = false;
            for (int p = 0; p < 26 && !hit; ++p) {
              double cand = node_id(c1 + probe[p][0], c2 + probe[p][1], c3 + probe[p][2], Nx, Ny);
              if (std::binary_search(lista.begin(), lista.end(), cand)) {
                found = cand;
                hit = true;
              }
            }
            M.nodes[v] = hit ? found : node_id(c1 + dx, c2 + dy, c3 + dz, Nx, Ny);
          } else {
            M.nodes[v] = node_id(c1, c2, c3, Nx, Ny);
          }
        }
  }
  M.nodes_red = M.nodes;
  std::sort(M.nodes_red.begin(), M.nodes_red.end());
  M.nodes_red.erase(std::unique(M.nodes_red.begin(), M.nodes_red.end()), M.nodes_red.end());
  M.vox_node.resize(M.num_vox);
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < M.num_vox; ++v)
    M.vox_node[v] = std::lower_bound(M.nodes_red.begin(), M.nodes_red.end(), M.nodes[v]) -
                    M.nodes_red.begin();
}

inline int64_t node_of(const Mesh& M, int x, int y, int z) {
  return M.vox_node[M.vox_map[M.cell(x, y, z)] - 1];
}

// first grid k holding both voxels with distinct nodes, or -1
inline int edge_grid(const Mesh& M, int x1, int y1, int z1, int x2, int y2, int z2) {
  for (int k = 0; k < M.G; ++k)
    if (M.at(k, x1, y1, z1) && M.at(k, x2, y2, z2)) {
      if (node_of(M, x1, y1, z1) != node_of(M, x2, y2, z2)) return k;
    }
  return -1;
}

void build_edges(Mesh& M, const std::vector<double>& sigma) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  // --- numbering (create_mapping_A{x,y,z}_v2.jl) ---
  // x: loops y, z, x ; y: z, x, y ; z: x, y, z (last index fastest). The edge grid of
  // every lattice cell is evaluated in parallel, then edges are numbered slab by slab of
  // the reference's outer loop: per-slab counts, their prefix sums, and each slab's
  // numbers in its inner loop order.
  const size_t Lx = (size_t)std::max(Nx - 1, 0) * Ny * Nz;
  const size_t Ly = (size_t)Nx * std::max(Ny - 1, 0) * Nz;
  const size_t Lz = (size_t)Nx * Ny * std::max(Nz - 1, 0);
  std::vector<int32_t> kx(Lx, -1), ky(Ly, -1), kz(Lz, -1);
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; ++z)
    for (int y = 0; y < Ny; ++y)
      for (int x = 0; x < Nx; ++x) {
        if (x + 1 < Nx) kx[((size_t)z * Ny + y) * (Nx - 1) + x] = edge_grid(M, x, y, z, x + 1, y, z);
        if (y + 1 < Ny) ky[((size_t)z * (Ny - 1) + y) * Nx + x] = edge_grid(M, x, y, z, x, y + 1, z);
        if (z + 1 < Nz) kz[((size_t)z * Ny + y) * Nx + x] = edge_grid(M, x, y, z, x, y, z + 1);
      }
  std::vector<int64_t> numx(Lx, -1), numy(Ly, -1), numz(Lz, -1);
  // number the cells of nslab slabs; visit(s, f) calls f(lattice cell) for slab s in order
  auto number = [](int nslab, const std::vector<int32_t>& kk, std::vector<int64_t>& num,
                   auto visit) -> int64_t {
    std::vector<int64_t> start((size_t)nslab + 1, 0);
#pragma omp parallel for schedule(static)
    for (int sl = 0; sl < nslab; ++sl) {
      int64_t c = 0;
      visit(sl, [&](size_t lc) { c += kk[lc] >= 0; });
      start[sl + 1] = c;
    }
    for (int sl = 0; sl < nslab; ++sl) start[sl + 1] += start[sl];
#pragma omp parallel for schedule(static)
    for (int sl = 0; sl < nslab; ++sl) {
      int64_t c = start[sl];
      visit(sl, [&](size_t lc) {
        if (kk[lc] >= 0) num[lc] = c++;
      });
    }
    return start[nslab];
  };
  M.m[0] = number(Ny, kx, numx, [&](int y, auto f) {
    for (int z = 0; z < Nz; ++z)
      for (int x = 0; x + 1 < Nx; ++x) f(((size_t)z * Ny + y) * (Nx - 1) + x);
  });
  M.m[1] = number(Nz, ky, numy, [&](int z, auto f) {
    for (int x = 0; x < Nx; ++x)
      for (int y = 0; y + 1 < Ny; ++y) f(((size_t)z * (Ny - 1) + y) * Nx + x);
  });
  M.m[2] = number(Nx, kz, numz, [&](int x, auto f) {
    for (int y = 0; y < Ny; ++y)
      for (int z = 0; z + 1 < Nz; ++z) f(((size_t)z * Ny + y) * Nx + x);
  });
  for (int d = 0; d < 3; ++d) {
    M.e_n1[d].assign(M.m[d], -1);
    M.e_n2[d].assign(M.m[d], -1);
    M.e_cell[d].assign(M.m[d], -1);
    M.e_mat[d].assign(M.m[d], 0);
    M.e_border1[d].assign(M.m[d], 0);
    M.e_border2[d].assign(M.m[d], 0);
    M.e_zs[d].assign(4 * M.m[d], 0);
  }
  auto G = [&](int k, int x, int y, int z) { return M.at(k, x, y, z); };
  // --- incidence, borders and surface-impedance counters
  //     (create_A_mats_and_find_borders_with_map_Zs.jl) ---
  // x edges (each edge's entries are written by its own iteration)
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; ++z)
    for (int y = 0; y < Ny; ++y)
      for (int x = 0; x + 1 < Nx; ++x) {
        size_t lc = ((size_t)z * Ny + y) * (Nx - 1) + x;
        int k = kx[lc];
        if (k < 0) continue;
        int64_t e = numx[lc];
        M.e_n1[0][e] = node_of(M, x, y, z);
        M.e_n2[0][e] = node_of(M, x + 1, y, z);
        M.e_cell[0][e] = (int64_t)lc;
        M.e_mat[0][e] = k + 1;
        int64_t* zs = &M.e_zs[0][4 * e];
        if (sigma[k] != 0) {
          // kind a = "x_xy" (neighbours along z), kind b = "x_zx" (along y)
          if (z == 0 || z == Nz - 1) {
            zs[0] += 1; zs[1] += 1;
          } else {
            if (!G(k, x, y, z - 1)) zs[0] += 1;
            if (!G(k, x + 1, y, z - 1)) zs[1] += 1;
            if (!G(k, x, y, z + 1)) zs[0] += 1;
            if (!G(k, x + 1, y, z + 1)) zs[1] += 1;
          }
          if (y == 0 || y == Ny - 1) {
            zs[2] += 1; zs[3] += 1;
          } else {
            if (!G(k, x, y - 1, z)) zs[2] += 1;
            if (!G(k, x + 1, y - 1, z)) zs[3] += 1;
            if (!G(k, x, y + 1, z)) zs[2] += 1;
            if (!G(k, x + 1, y + 1, z)) zs[3] += 1;
          }
        }
        if (x > 0) {
          if (!G(k, x - 1, y, z)) M.e_border1[0][e] = k + 1;
        } else {
          M.e_border1[0][e] = k + 1;
        }
        if (x + 2 == Nx) M.e_border2[0][e] = k + 1;
        else if (x + 2 <= Nx - 1 && !G(k, x + 2, y, z)) M.e_border2[0][e] = k + 1;
      }
  // y edges
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz; ++z)
    for (int x = 0; x < Nx; ++x)
      for (int y = 0; y + 1 < Ny; ++y) {
        size_t lc = ((size_t)z * (Ny - 1) + y) * Nx + x;
        int k = ky[lc];
        if (k < 0) continue;
        int64_t e = numy[lc];
        M.e_n1[1][e] = node_of(M, x, y, z);
        M.e_n2[1][e] = node_of(M, x, y + 1, z);
        M.e_cell[1][e] = (int64_t)lc;
        M.e_mat[1][e] = k + 1;
        int64_t* zs = &M.e_zs[1][4 * e];
        if (sigma[k] != 0) {
          // kind a = "y_xy" (along z), kind b = "y_yz" (along x)
          if (z == 0 || z == Nz - 1) {
            zs[0] += 1; zs[1] += 1;
          } else {
            if (!G(k, x, y, z - 1)) zs[0] += 1;
            if (!G(k, x, y + 1, z - 1)) zs[1] += 1;
            if (!G(k, x, y, z + 1)) zs[0] += 1;
            if (!G(k, x, y + 1, z + 1)) zs[1] += 1;
          }
          if (x == 0 || x == Nx - 1) {
            zs[2] += 1; zs[3] += 1;
          } else {
            if (!G(k, x - 1, y, z)) zs[2] += 1;
            if (!G(k, x - 1, y + 1, z)) zs[3] += 1;
            if (!G(k, x + 1, y, z)) zs[2] += 1;
            if (!G(k, x + 1, y + 1, z)) zs[3] += 1;
          }
        }
        if (y > 0) {
          if (!G(k, x, y - 1, z)) M.e_border1[1][e] = k + 1;
        } else {
          M.e_border1[1][e] = k + 1;
        }
        if (y + 2 == Ny) M.e_border2[1][e] = k + 1;
        else if (y + 2 <= Ny - 1 && !G(k, x, y + 2, z)) M.e_border2[1][e] = k + 1;
      }
  // z edges
#pragma omp parallel for schedule(static)
  for (int z = 0; z < Nz - 1; ++z)
    for (int y = 0; y < Ny; ++y)
      for (int x = 0; x < Nx; ++x) {
        size_t lc = ((size_t)z * Ny + y) * Nx + x;
        int k = kz[lc];
        if (k < 0) continue;
        int64_t e = numz[lc];
        M.e_n1[2][e] = node_of(M, x, y, z);
        M.e_n2[2][e] = node_of(M, x, y, z + 1);
        M.e_cell[2][e] = (int64_t)lc;
        M.e_mat[2][e] = k + 1;
        int64_t* zs = &M.e_zs[2][4 * e];
        if (sigma[k] != 0) {
          // kind a = "z_zx" (along x), kind b = "z_yz" (along y); the +1 side
          // tests the z-level of the first voxel for both counters, as the
          // reference does
          if (x == 0 || x == Nx - 1) {
            zs[0] += 1; zs[1] += 1;
          } else {
            if (!G(k, x - 1, y, z)) zs[0] += 1;
            if (!G(k, x - 1, y, z + 1)) zs[1] += 1;
            if (!G(k, x + 1, y, z)) zs[0] += 1;
            if (!G(k, x + 1, y, z)) zs[1] += 1;
          }
          if (y == 0 || y == Ny - 1) {
            zs[2] += 1; zs[3] += 1;
          } else {
            if (!G(k, x, y - 1, z)) zs[2] += 1;
            if (!G(k, x, y - 1, z + 1)) zs[3] += 1;
            if (!G(k, x, y + 1, z)) zs[2] += 1;
            if (!G(k, x, y + 1, z)) zs[3] += 1;
          }
        }
        if (z > 0) {
          if (!G(k, x, y, z - 1)) M.e_border1[2][e] = k + 1;
        } else {
          M.e_border1[2][e] = k + 1;
        }
        if (z + 2 == Nz) M.e_border2[2][e] = k + 1;
        else if (z + 2 <= Nz - 1 && !G(k, x, y, z + 2)) M.e_border2[2][e] = k + 1;
      }
}

struct SRec {
  int32_t fam;
  int64_t cell, node;
};

// Runs body(a, out) for the outer-loop slabs a = 0..n-1 in parallel, then appends their
// records in slab order: the same sequence as running the loop serially.
template <typename F>
void ordered_push(Mesh& M, int n, F body) {
  std::vector<std::vector<SRec>> per((size_t)std::max(n, 0));
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < n; ++a) body(a, per[a]);
  for (const auto& v : per)
    for (const auto& r : v) {
      M.s_fam.push_back(r.fam);
      M.s_cell.push_back(r.cell);
      M.s_node.push_back(r.node);
      M.ns_fam[r.fam] += 1;
    }
}

void build_surfaces(Mesh& M, const Ext& E) {
  const int Nx = M.Nx, Ny = M.Ny, Nz = M.Nz;
  auto G = [&](int k, int x, int y, int z) { return M.at(k, x, y, z); };
  auto any_other = [&](int k, bool ok, int x, int y, int z) {
    if (!ok) return false;
    for (int k2 = 0; k2 < M.G; ++k2)
      if (k2 != k && G(k2, x, y, z)) return true;
    return false;
  };
  auto rec = [&](std::vector<SRec>& out, int fam, size_t cell, int x, int y, int z) {
    out.push_back(SRec{fam, (int64_t)cell, node_of(M, x, y, z)});
  };
  // family 0 (reference "12", y-normal faces) on the Nx x (Ny+1) x Nz lattice
  auto c12 = [&](int x, int yf, int z) { return ((size_t)z * (Ny + 1) + yf) * Nx + x; };
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int z = 0; z < Nz; ++z) {  // y = 0
      int y = 0;
      for (int k = 0; k < M.G; ++k) {
        bool om = any_other(k, y + 1 <= Ny - 1, x, y + 1, z);
        if (G(k, x, y, z) && (!E.get(k, 1, M.cell(x, y, z)) || om)) {
          rec(out, 0, c12(x, y, z), x, y, z);
          break;
        }
      }
    }
  });
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int y = 1; y < Ny; ++y)
      for (int z = 0; z < Nz; ++z)
        for (int k = 0; k < M.G; ++k) {
          bool om = any_other(k, y + 1 <= Ny - 1, x, y + 1, z);
          if (G(k, x, y, z) && !G(k, x, y - 1, z) && (!E.get(k, 1, M.cell(x, y, z)) || om)) {
            rec(out, 0, c12(x, y, z), x, y, z);
            break;
          }
        }
  });
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int z = 0; z < Nz; ++z) {  // y = Ny-1, face Ny
      int y = Ny - 1;
      for (int k = 0; k < M.G; ++k) {
        bool om = any_other(k, y - 1 >= 0, x, y - 1, z);
        if (G(k, x, y, z) && (!E.get(k, 0, M.cell(x, y, z)) || om)) {
          rec(out, 0, c12(x, y + 1, z), x, y, z);
          break;
        }
      }
    }
  });
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int y = 0; y + 1 < Ny; ++y)
      for (int z = 0; z < Nz; ++z)
        for (int k = 0; k < M.G; ++k) {
          bool om = any_other(k, y - 1 >= 0, x, y - 1, z);
          if (G(k, x, y, z) && !G(k, x, y + 1, z) && (!E.get(k, 0, M.cell(x, y, z)) || om)) {
            if (!any_other(k, true, x, y + 1, z)) rec(out, 0, c12(x, y + 1, z), x, y, z);
            break;
          }
        }
  });
  // family 1 (reference "34", x-normal faces) on the (Nx+1) x Ny x Nz lattice
  auto c34 = [&](int xf, int y, int z) { return ((size_t)z * Ny + y) * (Nx + 1) + xf; };
  ordered_push(M, Ny, [&](int y, std::vector<SRec>& out) {
    for (int z = 0; z < Nz; ++z) {  // x = 0
      int x = 0;
      for (int k = 0; k < M.G; ++k) {
        bool om = any_other(k, x + 1 <= Nx - 1, x + 1, y, z);
        if (G(k, x, y, z) && (!E.get(k, 3, M.cell(x, y, z)) || om)) {
          rec(out, 1, c34(x, y, z), x, y, z);
          break;
        }
      }
    }
  });
  ordered_push(M, std::max(Nx - 1, 0), [&](int a, std::vector<SRec>& out) {
    const int x = a + 1;
    for (int y = 0; y < Ny; ++y)
      for (int z = 0; z < Nz; ++z)
        for (int k = 0; k < M.G; ++k) {
          bool om = any_other(k, x + 1 <= Nx - 1, x + 1, y, z);
          if (G(k, x, y, z) && !G(k, x - 1, y, z) && (!E.get(k, 3, M.cell(x, y, z)) || om)) {
            rec(out, 1, c34(x, y, z), x, y, z);
            break;
          }
        }
  });
  ordered_push(M, Ny, [&](int y, std::vector<SRec>& out) {
    for (int z = 0; z < Nz; ++z) {  // x = Nx-1, face Nx
      int x = Nx - 1;
      for (int k = 0; k < M.G; ++k) {
        bool om = any_other(k, x - 1 >= 0, x - 1, y, z);
        if (G(k, x, y, z) && (!E.get(k, 2, M.cell(x, y, z)) || om)) {
          rec(out, 1, c34(x + 1, y, z), x, y, z);
          break;
        }
      }
    }
  });
  ordered_push(M, std::max(Nx - 1, 0), [&](int x, std::vector<SRec>& out) {
    for (int y = 0; y < Ny; ++y)
      for (int z = 0; z < Nz; ++z)
        for (int k = 0; k < M.G; ++k) {
          bool om = any_other(k, x - 1 >= 0, x - 1, y, z);
          if (G(k, x, y, z) && !G(k, x + 1, y, z) && (!E.get(k, 2, M.cell(x, y, z)) || om)) {
            if (!any_other(k, true, x + 1, y, z)) rec(out, 1, c34(x + 1, y, z), x, y, z);
            break;
          }
        }
  });
  // family 2 (reference "56", z-normal faces) on the Nx x Ny x (Nz+1) lattice
  auto c56 = [&](int x, int y, int zf) { return ((size_t)zf * Ny + y) * Nx + x; };
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int y = 0; y < Ny; ++y) {  // z = 0
      int z = 0;
      for (int k = 0; k < M.G; ++k) {
        bool om = any_other(k, z + 1 <= Nz - 1, x, y, z + 1);
        if (G(k, x, y, z) && (!E.get(k, 5, M.cell(x, y, z)) || om)) {
          rec(out, 2, c56(x, y, z), x, y, z);
          break;
        }
      }
    }
  });
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int y = 0; y < Ny; ++y)
      for (int z = 1; z < Nz; ++z)
        for (int k = 0; k < M.G; ++k) {
          bool om = any_other(k, z + 1 <= Nz - 1, x, y, z + 1);
          if (G(k, x, y, z) && !G(k, x, y, z - 1) && (!E.get(k, 5, M.cell(x, y, z)) || om)) {
            rec(out, 2, c56(x, y, z), x, y, z);
            break;
          }
        }
  });
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int y = 0; y < Ny; ++y) {  // z = Nz-1, face Nz
      int z = Nz - 1;
      for (int k = 0; k < M.G; ++k) {
        bool om = any_other(k, z - 1 >= 0, x, y, z - 1);
        if (G(k, x, y, z) && (!E.get(k, 4, M.cell(x, y, z)) || om)) {
          rec(out, 2, c56(x, y, z + 1), x, y, z);
          break;
        }
      }
    }
  });
  ordered_push(M, Nx, [&](int x, std::vector<SRec>& out) {
    for (int y = 0; y < Ny; ++y)
      for (int z = 0; z + 1 < Nz; ++z)
        for (int k = 0; k < M.G; ++k) {
          bool om = any_other(k, z - 1 >= 0, x, y, z - 1);
          if (G(k, x, y, z) && !G(k, x, y, z + 1) && (!E.get(k, 4, M.cell(x, y, z)) || om)) {
            if (!any_other(k, true, x, y, z + 1)) rec(out, 2, c56(x, y, z + 1), x, y, z);
            break;
          }
        }
  });
}

}  // namespace

extern "C" {

// Builds the mesh; grids is G x Nx x Ny x Nz uint8 with x fastest per grid.
// dominant[k] != 0 marks conductor grids; sigma[k] is the conductivity.
void* peec_mesh_build(const uint8_t* grids, int G, int Nx, int Ny, int Nz,
                      const uint8_t* dominant, const double* sigma) {
  if (G <= 0 || Nx <= 0 || Ny <= 0 || Nz <= 0 || !grids) return nullptr;
  Mesh* M = new Mesh();
  M->G = G; M->Nx = Nx; M->Ny = Ny; M->Nz = Nz;
  size_t N = (size_t)Nx * Ny * Nz;
  M->g.assign(grids, grids + (size_t)G * N);
  // voxel numbering, x fastest (create_volumes_mapping.jl:10-22)
  M->vox_map.assign(N, 0);
  int64_t num = 0;
  for (size_t c = 0; c < N; ++c)
    for (int k = 0; k < G; ++k)
      if (M->g[(size_t)k * N + c]) {
        M->vox_map[c] = ++num;
        break;
      }
  M->num_vox = num;
  Ext E(G, (int)N);
  build_externals(*M, E);
  std::vector<uint8_t> dom(dominant, dominant + G);
  std::vector<double> sig(sigma, sigma + G);
  build_nodes(*M, E, dom);
  build_edges(*M, sig);
  build_surfaces(*M, E);
  // flatten into named arrays
  auto& I = M->iarr;
  I["vox_map"] = M->vox_map;
  I["vox_node"] = M->vox_node;
  I["counts"] = {M->num_vox, (int64_t)M->nodes_red.size(), M->m[0], M->m[1], M->m[2],
                 M->ns_fam[0], M->ns_fam[1], M->ns_fam[2]};
  std::vector<int64_t> n1, n2, cell, mat, b1, b2, zs;
  for (int d = 0; d < 3; ++d) {
    n1.insert(n1.end(), M->e_n1[d].begin(), M->e_n1[d].end());
    n2.insert(n2.end(), M->e_n2[d].begin(), M->e_n2[d].end());
    cell.insert(cell.end(), M->e_cell[d].begin(), M->e_cell[d].end());
    mat.insert(mat.end(), M->e_mat[d].begin(), M->e_mat[d].end());
    b1.insert(b1.end(), M->e_border1[d].begin(), M->e_border1[d].end());
    b2.insert(b2.end(), M->e_border2[d].begin(), M->e_border2[d].end());
    zs.insert(zs.end(), M->e_zs[d].begin(), M->e_zs[d].end());
  }
  I["edge_n1"] = n1; I["edge_n2"] = n2; I["edge_cell"] = cell; I["edge_mat"] = mat;
  I["edge_border1"] = b1; I["edge_border2"] = b2; I["edge_zs"] = zs;
  I["surf_node"] = M->s_node; I["surf_fam"] = M->s_fam; I["surf_cell"] = M->s_cell;
  M->darr["nodes"] = M->nodes;
  M->darr["nodes_red"] = M->nodes_red;
  return M;
}

// length of a named array (-1 if unknown); *is_double tells the element type
int64_t peec_mesh_len(void* h, const char* name, int* is_double) {
  Mesh* M = static_cast<Mesh*>(h);
  auto it = M->iarr.find(name);
  if (it != M->iarr.end()) { if (is_double) *is_double = 0; return (int64_t)it->second.size(); }
  auto jt = M->darr.find(name);
  if (jt != M->darr.end()) { if (is_double) *is_double = 1; return (int64_t)jt->second.size(); }
  return -1;
}

int peec_mesh_copy(void* h, const char* name, void* out) {
  Mesh* M = static_cast<Mesh*>(h);
  auto it = M->iarr.find(name);
  if (it != M->iarr.end()) {
    std::memcpy(out, it->second.data(), it->second.size() * sizeof(int64_t));
    return 0;
  }
  auto jt = M->darr.find(name);
  if (jt != M->darr.end()) {
    std::memcpy(out, jt->second.data(), jt->second.size() * sizeof(double));
    return 0;
  }
  return -1;
}

void peec_mesh_free(void* h) { delete static_cast<Mesh*>(h); }

}  // extern "C"
