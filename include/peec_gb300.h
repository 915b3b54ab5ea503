/*
 * peec_gb300.h -- C ABI of the GB300 FFT-PEEC solver path.
 *
 * The three reference entry points this library replaces (paths relative to the
 * Draco112358/Solver project) are
 *   compute_FFT_mutual_coupling_mats  src/lib/solverFFT/compute_FFT_mutual_coupling_mats.jl:1
 *   ComputeMatrixVectorFTT            src/lib/solverFFT/compute_Matrix_vector_fft.jl:1
 *   gmres_custom                      src/lib/solverFFT/gmres_custom.jl:1
 * and the per-port solve of the frequency loop FFT_solver_QS_S_type
 * (src/lib/solverFFT/FFT_solver_QS_S_type.jl:121-140, 237-262).
 *
 * Conventions: plain pointers and sizes; complex values are interleaved
 * (re, im) doubles, the layout of Julia ComplexF64 and C double _Complex; all
 * indices are 0-based (a Julia caller subtracts 1). Host buffers are
 * caller-owned and only read/written during the call. Every function returns
 * PEEC_OK or a negative PEEC_ERR_* code; peec_last_error() then describes it.
 * No C++ exception crosses this interface: an exhausted host allocation inside a
 * call returns PEEC_ERR_OOM, any other internal exception PEEC_ERR_STATE.
 * A context holds one geometry on one GPU with its own CUDA stream; contexts are
 * independent (no global state), so concurrent jobs use separate contexts.
 */
#ifndef PEEC_GB300_H
#define PEEC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PEEC_OK 0
#define PEEC_ERR_CUDA (-1)
#define PEEC_ERR_OOM (-2)
#define PEEC_ERR_CANCELLED (-3)
#define PEEC_ERR_TIMEOUT (-4)
#define PEEC_ERR_BADARG (-5)
#define PEEC_ERR_UNSUPPORTED (-6)
#define PEEC_ERR_STATE (-7)

/* arithmetic of the circulant convolutions (the sparse part is always FP64):
 * FP64, FP32, or float-float (hi + lo FP32 pairs, about 48 significant bits; the
 * FP64 data and spectra are split on load). Float-float has no counterpart in the
 * reference; it serves the refinement residuals of peec_solve_mixed, where GB300's
 * FP32 pipes are far faster than its FP64 ones. */
#define PEEC_PREC_FP64 0
#define PEEC_PREC_FP32 1
#define PEEC_PREC_FF 2

typedef struct peec_ctx peec_ctx;

/* ABI version (major*100 + minor). */
int peec_version(void);

/* Create / destroy a context on CUDA device `device`. */
int peec_ctx_create(peec_ctx** out, int device);
void peec_ctx_destroy(peec_ctx* ctx);
/* Last error message of the context (never NULL). */
const char* peec_last_error(const peec_ctx* ctx);

/*
 * Geometry and topology: the content of the reference's incidence_selection and
 * expansions dictionaries (mesher_FFT.jl:36-84, create_mapping_Gamma_no_rep.jl:381-419).
 *   Nx, Ny, Nz      voxel grid
 *   mx, my, mz      edges per direction; edges are ordered x, then y, then z
 *   edge_cell[m]    lattice cell of each edge in its direction lattice
 *                   ((Nx-1)xNyxNz, Nx(Ny-1)Nz, NxNy(Nz-1); x fastest) -- the row of
 *                   its 1 in mat_map_Lp[c,1]
 *   edge_n1/n2[m]   the nodes with A(e,n1) = -1, A(e,n2) = +1
 *   ns              surfaces; surf_fam[s] in 0..2 is the face family (reference
 *                   families 12, 34, 56), surf_cell[s] its cell in the family
 *                   lattice (Nx(Ny+1)Nz, (Nx+1)NyNz, NxNy(Nz+1)) -- the row of its 1
 *                   in exp_P[f,f]; surf_node[s] the node of its 1 in Gamma
 *   n               nodes
 * The cross-family exp_P blocks are implied by this placement (their lattice rows
 * are fixed functions of the family cells), so they are not passed.
 * Limits (PEEC_ERR_UNSUPPORTED beyond them): m + ns + n and 2m + 1 fit in int32;
 * every circulant length (the power of two at or above about twice the lattice
 * extent along its axis) is at most 8192, so no axis is longer than 4096 cells.
 */
int peec_set_topology(peec_ctx* ctx, int Nx, int Ny, int Nz, int64_t mx, int64_t my, int64_t mz,
                      const int64_t* edge_cell, const int64_t* edge_n1, const int64_t* edge_n2,
                      int64_t ns, const int32_t* surf_fam, const int64_t* surf_cell,
                      const int64_t* surf_node, int64_t n);

/*
 * Topology of a mesh without voxel lattices (the dense RIS solver,
 * solverRis/iter_solver_QS_S_type.jl): the edges' end nodes (A, -1 at n1 and +1 at
 * n2, edges ordered x, y, z with mx, my, mz of each) and the surfaces' nodes (Gamma,
 * one node per surface). The operator then needs peec_set_dense; the circulant entry
 * points (peec_fill, peec_set_rows, the Rcc rows, peec_adjoint) return PEEC_ERR_STATE.
 */
int peec_set_incidence(peec_ctx* ctx, int64_t mx, int64_t my, int64_t mz,
                       const int64_t* edge_n1, const int64_t* edge_n2, int64_t ns,
                       const int64_t* surf_node, int64_t n);

/*
 * Dense operator blocks (ComputeMatrixVectorRis, solverRis/compute_matrix_vector.jl:1-33):
 * Lp_x (mx x mx), Lp_y (my x my), Lp_z (mz x mz) and P (ns x ns), real, column-major
 * (Lp_data[:Lp_x], ..., P_data[:P]). Each operator application multiplies them with the
 * edge currents and surface charges (FP64, or an FP32 copy in PEEC_PREC_FP32), Lp without
 * its diagonal; the frequency state (peec_set_frequency) takes DZ = Z_self + jw diag(Lp),
 * the denominator of the RIS solver's invZ, so that the first block row is
 * jw Lp I + Z_self I + A Phi and the preconditioner is the RIS solver's. Replaces a
 * circulant operator set before; peec_fill / peec_set_rows replace the dense one.
 */
int peec_set_dense(peec_ctx* ctx, const double* Lp_x, const double* Lp_y, const double* Lp_z,
                   const double* P);

/*
 * Per-edge data from which the device forms each frequency's edge impedances DZ
 * (FFT_solver_QS_S_type.jl:105-114, compute_Z_self.jl): R4 and Cd4 the resistances and
 * capacitances of the four edge halves (m x 4, row-major; diagonals["R"], ["Cd"]), Lp_self
 * the Lp self terms (diagonals["Lp"]), Zs0 the real surface-impedance base (the
 * frequency's Zs is escal_R * Zs0 * sqrt(w / escal_freq)) and the nse surface edges.
 * Copied; used by peec_set_frequency_device.
 */
int peec_set_edge_state(peec_ctx* ctx, const double* R4, const double* Cd4, const double* Lp_self,
                        const double* Zs0, const int64_t* surface_edges, int64_t nse,
                        double escal_R, double escal_freq);

/*
 * One frequency's state formed on the device: DZ from the edge data
 * (peec_set_edge_state) -- Z_self, the surface-impedance selection on surface edges and
 * jw Lp_self, as the reference forms them on the host each frequency -- and SS assembled
 * and factorised in the pattern of peec_lu_refactor_setup (Yle with that set-up's
 * pattern). The caller passes only w and Yle. Keeps the captured graphs, like
 * peec_set_frequency_refactor. No counterpart in the reference.
 */
int peec_set_frequency_device(peec_ctx* ctx, double w, int64_t yle_nnz, const int64_t* yle_row,
                              const int64_t* yle_col, const double* yle_val);

/*
 * The dense retarded operator (the RIS solver with QS_Rcc_FW == 2,
 * iter_solver_QS_S_type.jl:39-59): the centre distances of the blocks peec_set_dense
 * installed (Lp_data[:Rx], [:Ry], [:Rz], P_data[:R_cc]; real, column-major, zero on the
 * diagonal). From then on the operator multiplies with the blocks times exp(-j beta R)
 * of the frequency set by peec_set_dense_rcc_frequency (beta = 2 pi f sqrt(eps0 mu0), f
 * in Hz), formed on the device (FP64 and an FP32 copy) in place. All four pointers NULL
 * (or peec_set_dense) return the context to the quasi-static blocks; with distances on the
 * device (peec_ris_fill), a later peec_set_dense_rcc_frequency returns it to the retarded
 * operator.
 */
int peec_set_dense_rcc(peec_ctx* ctx, const double* Rx, const double* Ry, const double* Rz,
                       const double* Rcc);
int peec_set_dense_rcc_frequency(peec_ctx* ctx, double beta);

/*
 * The dense RIS matrices filled on the device from the bodies' vertex coordinates:
 * replaces calcola_Lp (sharedRis/calcola_Lp.jl:1-97) and calcola_P (sharedRis/calcola_P.jl:
 * 1-47), and takes the place of peec_set_dense + peec_set_pdiag (+ peec_set_dense_rcc when
 * distances != 0). Needs the topology of peec_set_incidence (mx, my, mz, ns).
 *   vol_coords   m x 24 row-major: volumi[:coordinate], eight vertices (x, y, z) per volume
 *   vol_S        m: volumi[:S], the cross-sections
 *   vol_centres  m x 3: volumi[:centri] (read when distances != 0)
 *   escal_Lp     escalings[:Lp]
 *   surf_ends    ns x 12 row-major: superfici["estremi_celle"], four vertices per surface
 *   surf_S       ns: superfici["S"]
 *   surf_centres ns x 3: superfici["centri"] (read when distances != 0)
 *   escal_P      escalings[:P]
 * Lp blocks: Compute_Lp_Self on the diagonal, 1e-7 / (S_m S_n) * integral * escal_Lp off it
 * (Song_improved_Ivana_strategy2); P: integral / (4 pi eps0 S_m S_n) * escal_P
 * (Song_P_improved_Ivana_strategy), the diagonal included; distances |c_m - c_n|
 * (calculate_Rx/_Ry/_Rz, calculate_R_cc!). Either group of pointers may be NULL: its
 * blocks are left as they are. *nonfinite (may be NULL) gets the count of non-finite
 * entries (the reference's closed forms give NaN in a few degenerate configurations).
 */
int peec_ris_fill(peec_ctx* ctx, const double* vol_coords, const double* vol_S,
                  const double* vol_centres, double escal_Lp, const double* surf_ends,
                  const double* surf_S, const double* surf_centres, double escal_P, int distances,
                  int64_t* nonfinite);

/*
 * A dense block back to the host: block 0..2 = Lp_x, Lp_y, Lp_z, 3 = P; what 0 = the
 * matrix (n x n, column-major), 1 = its centre distances, 2 = its diagonal (n values).
 * No counterpart in the reference (its matrices live on the host).
 */
int peec_dense_get(peec_ctx* ctx, int block, int what, double* out);

/* P self terms diag(P) per surface (diagonals["P"]); invP = 1 ./ diagP. */
int peec_set_pdiag(peec_ctx* ctx, const double* diagP);

/*
 * Generating rows of the nine circulant blocks, escaled, on the reference
 * lattices (column-major, x fastest), in the order
 *   Lpx, Lpy, Lpz, p12_se, p34_se, p56_se, p1234, p1256, p3456
 * i.e. the first row of each block before store_circulant_fft
 * (compute_FFT_mutual_coupling_mats.jl:52-125; Lp self entry already zeroed).
 * Builds the device spectra. Replaces passing FFTCLp / FFTCP.
 */
int peec_set_rows(peec_ctx* ctx, const double* const rows[9]);

/*
 * GPU fill of the nine generating rows and their spectra -- the drop-in for
 * compute_FFT_mutual_coupling_mats with QS_Rcc_FW == 1. origin is the mesh
 * origin (unscaled, as the reference passes it), s* the escaled cell sizes.
 * rows_out may be NULL, or hold nine host buffers (or NULL entries) that receive
 * the rows. Every branch of the reference's integral dispatch is evaluated,
 * the far-field (suppressed) ones included. Returns PEEC_ERR_UNSUPPORTED if an
 * entry comes out non-finite (degenerate cell sizes).
 */
int peec_fill(peec_ctx* ctx, const double origin[3], double sx, double sy, double sz,
              double escal_Lp, double escal_P, double* const rows_out[9]);

/*
 * Retarded operator (QS_Rcc_FW == 2, "Rcc"). Replaces compute_rows_Rcc_Lp /
 * compute_rows_Rcc_P (compute_FFT_mutual_coupling_mats.jl:17-27) and the per-frequency
 * compute_Circulant_Lp_Rcc / compute_Circulant_P_sup_Rcc calls of
 * FFT_solver_QS_S_type.jl:61-93.
 *
 * peec_fill_rcc: GPU fill of the quasi-static parts of the nine Rcc rows, escaled, in
 * the peec_set_rows order: the Lp rows through the Rcc path's own integral dispatch
 * (compute_Lp_Voxels_QS.jl:8-397, Lp self entries zeroed), the P rows with the face
 * types that path passes (the block indices, compute_rows_Rcc_P.jl:47-52). The rows stay
 * on the device; rows_out as for peec_fill. An Lp entry in that dispatch's orthogonal
 * surface-surface case, which the reference cannot evaluate (its call passes an
 * interval where the integral takes a coordinate, compute_Lp_Voxels_QS.jl:330-352),
 * returns PEEC_ERR_UNSUPPORTED.
 * peec_set_rows_rcc: the same rows from the host (shared-fill parity runs), with the
 * mesh geometry the centre distances need.
 * peec_set_rcc_frequency: the spectra at freq_hz (Hz, unscaled): each row times
 * exp(-i beta R), beta = 2 pi f sqrt(eps0 mu0), R the distance between centres (voxel
 * centres for Lp, QS face centres for P; compute_Voxels_Rcc.jl, compute_P_vox_Rcc.jl).
 * From then on operator applications, solves and port right-hand sides use the Rcc
 * operator, until peec_set_rows / peec_fill install QS spectra again.
 */
int peec_fill_rcc(peec_ctx* ctx, const double origin[3], double sx, double sy, double sz,
                  double escal_Lp, double escal_P, double* const rows_out[9]);
int peec_set_rows_rcc(peec_ctx* ctx, const double* const rows[9], const double origin[3],
                      double sx, double sy, double sz);
int peec_set_rcc_frequency(peec_ctx* ctx, double freq_hz);

/*
 * Per-frequency state (FFT_solver_QS_S_type.jl:105-119): scaled angular
 * frequency w, DZ[m] (complex), Yle as COO (complex values), and the sparse LU
 * factors of SS with Pr*diag(row_scale)*SS*Pc = L*U in CSR form (L lower, U upper;
 * both include their diagonal), perm_r / perm_c as in SuperLU (row i goes to row
 * perm_r[i]; column i to column perm_c[i]). row_scale may be NULL (no scaling; for
 * UMFPACK factors pass F.Rs).
 */
int peec_set_frequency(peec_ctx* ctx, double w, const double* DZ, int64_t yle_nnz,
                       const int64_t* yle_row, const int64_t* yle_col, const double* yle_val,
                       const int64_t* L_ptr, const int64_t* L_col, const double* L_val,
                       const int64_t* U_ptr, const int64_t* U_col, const double* U_val,
                       const int64_t* perm_r, const int64_t* perm_c, const double* row_scale);

/*
 * Device factorisation of SS at later frequencies (replaces the per-frequency lu(SS) of
 * FFT_solver_QS_S_type.jl:118-119 after the first frequency). SS's structure does not
 * depend on the frequency, so the factors of one host factorisation (installed by
 * peec_set_frequency) fix the pattern and the pivot order:
 * peec_lu_refactor_setup: builds the plan from the installed factors and the Yle pattern
 * (COO, values not read).
 * peec_set_frequency_refactor: DZ and Yle as for peec_set_frequency (Yle with the same
 * pattern), then SS assembled and factorised on the device (one launch per level of L),
 * no host factors. A zero or non-finite pivot returns PEEC_ERR_UNSUPPORTED (factorise that
 * frequency on the host); a later peec_set_frequency drops the plan.
 */
int peec_lu_refactor_setup(peec_ctx* ctx, int64_t yle_nnz, const int64_t* yle_row,
                           const int64_t* yle_col);
int peec_set_frequency_refactor(peec_ctx* ctx, double w, const double* DZ, int64_t yle_nnz,
                                const int64_t* yle_row, const int64_t* yle_col,
                                const double* yle_val);

/*
 * Voxel mesher on the GPU (mesher_FFT.jl's topology: create_volumes_mapping.jl,
 * create_Grids_externals.jl, create_nodes_ref.jl, create_mapping_A{x,y,z}_v2.jl,
 * create_A_mats_and_find_borders_with_map_Zs.jl, create_mapping_Gamma_no_rep.jl), no
 * context needed. grids: G x Nx x Ny x Nz bytes (nonzero: occupied), x fastest per grid;
 * dominant[k] != 0 for conductor grids; sigma[k] the conductivities. Runs on `device`
 * (the caller's current device is restored); 27 Nx Ny Nz must fit in int32. Returns a
 * handle or NULL (the reason in *err_out when err_out is not NULL). The handle's arrays
 * (int64 unless noted): "vox_map" (per cell, 1-based voxel number, 0 empty), "vox_node",
 * "counts" (voxels, nodes, x/y/z edges, surfaces per family), "edge_n1", "edge_n2",
 * "edge_cell", "edge_mat", "edge_border1", "edge_border2", "edge_zs" (4 per edge),
 * "surf_node", "surf_fam", "surf_cell", "nodes" and "nodes_red" (double). Lengths by
 * peec_mesh_gpu_len (-1: no such array; *is_double set), contents by peec_mesh_gpu_copy.
 */
void* peec_mesh_gpu_build(const uint8_t* grids, int G, int Nx, int Ny, int Nz,
                          const uint8_t* dominant, const double* sigma, int device,
                          const char** err_out);
int64_t peec_mesh_gpu_len(void* mesh, const char* name, int* is_double);
int peec_mesh_gpu_copy(void* mesh, const char* name, void* out);
void peec_mesh_gpu_free(void* mesh);

/* y = M^-1 K x (ComputeMatrixVectorFTT); x, y host, length N = m + ns + n complex. */
int peec_matvec(peec_ctx* ctx, const double* x, double* y, int precision);
/* same on device pointers (complex double) */
int peec_matvec_dev(peec_ctx* ctx, const void* x, void* y, int precision);

/*
 * Right-hand side of port (n1, n2): M^-1 [0; 0; is] with is = +Is at n1, -Is at
 * n2 (precond_3_3_Kt_fft!, FFT_solver_QS_S_type.jl:124-127,237-262). tn host, N.
 */
int peec_port_rhs(peec_ctx* ctx, int64_t n1, int64_t n2, double Is, double* tn);

/*
 * Householder GMRES with the reference's MATLAB semantics (gmres_custom):
 * b, x_inout host (N complex); restarted = 0 runs one cycle of maxit inner steps
 * (the reference's only call form), restarted = 1 runs maxit cycles of `restart`
 * steps. flag: 0 converged, 1 not converged, 3 stagnation, 99 stopped.
 * iter[2] = (outer, inner). resvec receives up to resvec_cap norms; *nres their
 * count. relres is the left-preconditioned relative residual.
 */
int peec_gmres(peec_ctx* ctx, const double* b, double* x_inout, double tol, int maxit,
               int restarted, int restart, int precision, int* flag, double* relres,
               int* iter, double* resvec, int resvec_cap, int* nres);

/*
 * Mixed-precision solve: GMRES inner solves on the FP32-convolution operator inside
 * iterative refinement with FP64 vectors, to relative residual tol. The refinement
 * residuals b - A x use the operator in the residual precision (float-float by
 * default, see peec_set_residual_precision). inner_tol / inner_maxit bound each
 * inner solve, max_outer the refinements. outer_out / inner_total report the work;
 * relres the final relative residual. No counterpart in the reference (which solves
 * with FP64 GMRES only, FFT_solver_QS_S_type.jl:140).
 */
int peec_solve_mixed(peec_ctx* ctx, const double* b, double* x_inout, double tol,
                     double inner_tol, int inner_maxit, int max_outer, int* flag,
                     double* relres, int* outer_out, int* inner_total);

/*
 * Gradient of a port voltage in per-voxel parameters, by reciprocity. The operator's
 * edge block is diagonal in a voxel parameter (conductivity: the resistance halves
 * and the surface impedance, compute_diagonals.jl:10-12, compute_Zs_with_indices.jl:
 * 27-32) and the unpreconditioned matrix satisfies K^T = D1 K D2 with diagonal D1,
 * D2, so the port's adjoint solution is its forward solution rescaled. With I =
 * x[0:m] the edge currents of the port solution x (N complex, host), returns per voxel
 *   g[v] = (2/Is) * ( sum_{e: v1[e]=v} d1[e] I_e^2 + sum_{e: v2[e]=v} d2[e] I_e^2 ),
 * the derivative of the port voltage 2(phi_n1 - phi_n2) with respect to the parameter
 * of voxel v. d1 / d2 (m complex, host) are the derivatives of the edge impedance DZ_e
 * with respect to the parameter of the edge's first / second voxel v1[e] / v2[e]
 * (int32, -1: none). g: nvox complex (host). The reference has no gradient; this is
 * the device half of the adjoint configuration (solver_gb300/gradient.py).
 */
int peec_adjoint(peec_ctx* ctx, const double* x, const int32_t* v1, const int32_t* v2,
                 const double* d1, const double* d2, double Is, int64_t nvox, double* g);

/*
 * Self-test of the bounded-wait failure path: runs the synchronisation-free
 * triangular-solve kernel on a two-row system whose second row depends on a row that
 * is never solved, so its dependency wait gives up after its poll limit (about 50 ms)
 * and records the error word. Returns PEEC_ERR_TIMEOUT when that path works (the
 * expected result); the context stays usable. No counterpart in the reference.
 */
int peec_check_wait_limit(peec_ctx* ctx);

/*
 * Work split of the LU solves inside the operator: rows of connected components of
 * the factors with at most max_rows rows (0..512, default 512) are solved per warp, the
 * components of at most 32 rows packed several to a warp, each warp's rows, entries and
 * right-hand sides first loaded into shared memory; all other rows by the
 * synchronisation-free global scheme. Both give the same results to rounding; 0 routes
 * every row through the global scheme. Takes effect at once. No counterpart in the
 * reference (UMFPACK solves, FFT_solver_QS_S_type.jl:119).
 */
int peec_set_lu_component_max(peec_ctx* ctx, int max_rows);

/*
 * Arithmetic of the refinement residuals of peec_solve_mixed: PEEC_PREC_FF (default)
 * or PEEC_PREC_FP64. No counterpart in the reference.
 */
int peec_set_residual_precision(peec_ctx* ctx, int precision);

/*
 * Cooperative cancellation (is_stop_requested, solver_start.jl:370-374): a host
 * int the caller may set to nonzero at any time; the solvers poll it between
 * Krylov steps and return PEEC_ERR_CANCELLED (gmres flag 99). NULL disables.
 */
int peec_set_stop_flag(peec_ctx* ctx, volatile int* flag);

/*
 * The GMRES iterations of peec_gmres and of peec_solve_mixed's inner solves run on the
 * device: the scalar work of an iteration (reflector heads, Givens rotations, the
 * least-squares right-hand side, the residual estimate) is one FP64 kernel, and a CUDA
 * graph with a WHILE conditional node repeats the iteration until the estimate reaches
 * the tolerance or the restart cycle is full, with no host synchronisation in between.
 * The host keeps the reference's control flow (gmres_custom.jl:129-250): the checks on
 * the true residual, stagnation, restarts. on = 0 runs the same kernels one iteration
 * per host round trip instead (the same results, bit for bit); the stop flag is then
 * polled every iteration rather than every run of iterations. Default 1.
 * No counterpart in the reference.
 */
int peec_set_device_loop(peec_ctx* ctx, int on);

/*
 * Since the context was created: launches of the device-loop graph, and the GMRES
 * iterations they ran.
 */
int peec_device_loop_stats(const peec_ctx* ctx, int64_t* graph_launches, int64_t* iterations);

/*
 * Timing of the last peec_matvec / peec_matvec_dev call on the context stream
 * (CUDA events): total, convolutions, sparse epilogue + LU, in milliseconds.
 */
int peec_last_timing(peec_ctx* ctx, double* total_ms, double* conv_ms, double* sparse_ms);

/* The CUDA stream (cudaStream_t) all work of the context is issued on. */
void* peec_stream(const peec_ctx* ctx);

/* Number of lattice families of the operator (6: three face families, three edge
 * directions). */
int peec_conv_count(const peec_ctx* ctx);
/*
 * Family i: circulant grid L[3], lattice extents dims[3], whether it is present in
 * the geometry (*active) and its kind (0 = face family of P, 1 = edge family of Lp).
 * Face families share one grid and the six P spectra (three real, three complex);
 * each edge family has one real spectrum on its own grid.
 */
int peec_conv_info(const peec_ctx* ctx, int i, int* L, int* dims, int* active, int* kind);
/*
 * Profiling: the FP32 z-pass forms the autotuner picked for this context's grids, and the
 * times it measured (ms per z pass, mean of three after a warm-up; -1 where a form was not
 * a candidate). Forms: 0 register-direct kernels on the full-form spectra, 1 register-direct
 * on the y/z-folded FP32 spectra (Lx(Ly/2+1)(Lz/2+1) values per block), 2 staged
 * (persistent CTAs, each tile's pencils brought into shared memory by bulk asynchronous
 * copies while the previous tile computes, y/z-folded spectra; the edge families in one
 * launch). choice = {face form, edge form, edge radix plan}; face_ms[form];
 * edge_ms[plan * 3 + form]. The tuner runs when the spectra are built (peec_fill,
 * peec_set_rows) and caches its choice per device and grids. No counterpart in the
 * reference (it plans FFTW with MEASURE, FFT_solver_QS_S_type.jl:17-53).
 */
int peec_zpass_tuning(const peec_ctx* ctx, int choice[3], double face_ms[3], double edge_ms[6]);
/*
 * Pins the FP32 z-pass forms (face, edge: 0..2 as above; edge_plan 0..1) in place of the
 * tuner's choice, until the next peec_fill / peec_set_rows. A form a grid cannot take
 * (partial 16-column tiles, too few z points) runs as form 0; peec_zpass_tuning reports
 * the form that runs. For tests and for callers who fix the kernels. No counterpart in the
 * reference.
 */
int peec_set_zpass_forms(peec_ctx* ctx, int face, int edge, int edge_plan);

/*
 * Runs `iters` operator applications on an internal vector and reports the mean
 * per-application device time of each pass class, measured with CUDA events on the
 * context stream: ms[0] x-forward (gather + FFT), ms[1] y-forward FFTs, ms[2] z
 * passes (FFT, spectral product, inverse FFT), ms[3] y-inverse FFTs, ms[4]
 * x-inverse (FFT + scatter), ms[5] sparse epilogue and LU solve, ms[6] whole
 * application.
 */
int peec_profile_matvec(peec_ctx* ctx, int precision, int iters, double* ms);

/*
 * Batched inner products of Krylov vectors (the reductions of the GMRES reflector
 * updates, gmres_custom.jl:112-127): out[c] = sum_i conj(U[i + c*ldu]) * v[i] for
 * c < k. U, v, out are device pointers to complex doubles; runs on the context
 * stream and returns after the result is in `out`. Partial sums go to scratch
 * owned by the context (grown on demand).
 */
int peec_multidot(peec_ctx* ctx, const void* U, int64_t ldu, const void* v, int64_t N, int k,
                  void* out);

/*
 * Allocation-free variant of peec_multidot, for callers that cannot allocate
 * device memory when they need the reductions (a runtime whose device memory is
 * owned by its own pool, or a loop that must not take the implicit device
 * synchronisation of cudaMalloc/cudaFree). It has no counterpart in the reference.
 * No context; U, v, out are device pointers to complex doubles on the current
 * device; `stream` is a cudaStream_t (NULL = legacy default stream); returns after
 * `out` holds the result.
 * Scratch: a fixed file-scope device array of PEEC_NOALLOC_MAX_K x 304 complex
 * doubles (1.25 MB), resident on every GPU that loads the library until the
 * process exits. k > PEEC_NOALLOC_MAX_K is rejected with PEEC_ERR_BADARG; any N
 * is accepted. Set-up: the first call in each CUDA context of a device looks up
 * the array's device address; under lazy module loading that first call also
 * loads the library's device code onto the device, which is when the runtime
 * places the array (1.25 MB, possibly with a synchronisation). A caller whose
 * pool later takes all device memory should make one small call first, and that
 * first call should come before any stream capture. A failure there returns
 * PEEC_ERR_OOM or PEEC_ERR_CUDA with a message. After a device reset the next
 * call looks the address up again. The call synchronises its stream before it
 * returns. All calls on a device share the array and take it in turn: a
 * per-device lock is held from launch to completion, so calls from several
 * threads or streams are serialised rather than racing on the array. Calls no
 * cudaMalloc/cudaFree and no allocating library routine.
 */
#define PEEC_NOALLOC_MAX_K 256
int peec_multidot_noalloc(const void* U, int64_t ldu, const void* v, int64_t N, int k,
                          void* out, void* stream);

/* Counters: kernel launches issued by the context since creation. */
int64_t peec_launch_count(const peec_ctx* ctx);

/* Vector sizes of the current topology: m, ns, n (N = m+ns+n). */
int peec_sizes(const peec_ctx* ctx, int64_t* m, int64_t* ns, int64_t* n);

#ifdef __cplusplus
}
#endif

#endif /* PEEC_GB300_H */
