/*
 * dgx.h -- C ABI of the GB300-native explicit DG residual-and-update path.
 *
 * This library replaces the hot path of dgfem (GaleAxiom/Discontinuous-Galerkin-FEM):
 * the compressible Euler / Navier-Stokes residual (volume flux integral, Rusanov face
 * flux lifted to element modes, SIPG-style viscous terms), the block inverse mass
 * matrix and the SSP-RK3 stage update.  Each entry point names the dgfem interface it
 * replaces (paths inside the dgfem project).
 *
 * Conventions
 *  - Plain pointers and sizes only.  Functions return DGX_OK (0) or a negative status;
 *    dgx_last_error() gives the message of the last failure on the calling thread.
 *  - A state is double[n_elements][n_basis][4] (rho, rho*u, rho*v, E): dgfem's flat
 *    DGSolution index elem*Np*4 + i*4 + v (src/core/solution.cpp:143-145), i.e. the
 *    per-element Np x 4 matrices of `std::vector<Eigen::MatrixXd>` stored row-major.
 *  - Functions with a `stream` argument take DEVICE pointers and are stream-ordered
 *    (stream is a cudaStream_t; NULL = legacy default stream).  `_host` variants take
 *    host pointers and synchronise before returning.
 *  - A context is not thread-safe: use one per thread (dgfem's assembler is not
 *    re-entrant either, src/solver/assembler.cpp:143-150).
 *  - There is no CPU fallback: every compute entry point fails with DGX_ERR_CUDA when
 *    no sm_103 device is present.
 */
#ifndef DGX_H
#define DGX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGX_OK 0
#define DGX_ERR_INVALID (-1)   /* std::invalid_argument in dgfem */
#define DGX_ERR_RUNTIME (-2)   /* std::runtime_error in dgfem */
#define DGX_ERR_RANGE (-3)     /* std::out_of_range in dgfem */
#define DGX_ERR_CUDA (-4)      /* CUDA failure or no usable GPU */
#define DGX_ERR_NONFINITE (-5) /* non-finite or non-positive state detected */
#define DGX_ERR_TIMEOUT (-6)   /* a bounded wait inside a kernel gave up (dgx_step_status) */

/* DGX_BASIS_LEGENDRE: LegendreBasis (src/basis/legendre.cpp), the basis of quadrilateral
 * meshes (DGSpace::create_basis, src/core/space.cpp:307-319). */
enum { DGX_BASIS_MONOMIAL = 0, DGX_BASIS_DUBINER = 1, DGX_BASIS_LEGENDRE = 2 };
enum { DGX_EULER = 0, DGX_NAVIER_STOKES = 1 };
/* DGX_FP64: FP64 arithmetic and state (the plain form).  DGX_MIXED: FP32 flux and
 * contraction arithmetic, FP64 geometry, M^-1 and RK3 state.  DGX_DF64: the FP64 path's
 * algorithm and FP64 state with the residual computed in double-float arithmetic (pairs of
 * FP32 numbers, about 48 significant bits) on the FP32 pipe; no dgfem counterpart. */
enum { DGX_FP64 = 0, DGX_MIXED = 1, DGX_DF64 = 2 };
/* BCTypeEuler, include/dgfem/boundary/conditions.hpp:27-32 */
enum { DGX_BC_FAR_FIELD = 0, DGX_BC_SLIP_WALL = 1, DGX_BC_NO_SLIP_WALL = 2, DGX_BC_PERIODIC = 3 };

typedef struct dgx_mesh dgx_mesh;
typedef struct dgx_ctx dgx_ctx;

/* Weak form + space parameters.
 * Replaces DGSpace(type, order) (include/dgfem/core/space.hpp:27),
 * EulerWeakFormulation(gamma) (include/dgfem/weak_forms/euler_weak_formulation.hpp:18) and
 * NavierStokesWeakFormulation(gamma, mu, Pr, sigma0)
 * (include/dgfem/weak_forms/navier_stokes_weak_formulation.hpp:19-20). */
typedef struct {
    int order;      /* polynomial order p, 1..4 (triangles and quadrilaterals) */
    int basis;      /* triangles: DGX_BASIS_MONOMIAL (dgfem's default) or DGX_BASIS_DUBINER;
                       quadrilaterals: DGX_BASIS_LEGENDRE */
    int physics;    /* DGX_EULER or DGX_NAVIER_STOKES */
    int precision;  /* DGX_FP64, DGX_MIXED or DGX_DF64 */
    double gamma;   /* 1.4 */
    double mu;      /* dynamic viscosity (Navier-Stokes) */
    double prandtl; /* Prandtl number (Navier-Stokes) */
    double sigma0;  /* SIPG penalty prefactor (Navier-Stokes) */
} dgx_params;

const char* dgx_last_error(void);
const char* dgx_version(void);

/* ---------------------------------------------------------------- mesh (host) */

/* DGMesh(vertices, elements, element_tags, boundary_tags, boundary_edges),
 * include/dgfem/core/mesh.hpp:31-33, src/core/mesh.cpp:18-51, 312-402.
 * vertices: [n_vertices][2]; elements: [n_elements][3] vertex ids (triangles);
 * tag_names/tag_ids: the boundary_tags map; boundary_edges: [n_edges][3] = (tag, v1, v2). */
int dgx_mesh_create(int n_vertices, const double* vertices, int n_elements, const int* elements,
                    int n_tags, const char* const* tag_names, const int* tag_ids,
                    int n_boundary_edges, const int* boundary_edges, dgx_mesh** out);
/* The same for vertices_per_element = 3 (triangles) or 4 (bilinear quadrilaterals,
 * counter-clockwise; DGMesh picks "quad" from the element matrix's 4 columns,
 * src/core/mesh.cpp:23-35).  elements: [n_elements][vertices_per_element]. */
int dgx_mesh_create_nv(int vertices_per_element, int n_vertices, const double* vertices, int n_elements,
                       const int* elements, int n_tags, const char* const* tag_names, const int* tag_ids,
                       int n_boundary_edges, const int* boundary_edges, dgx_mesh** out);
/* vertices per element of a mesh: 3 or 4 (DGMesh::get_element_type) */
int dgx_mesh_vertices_per_element(const dgx_mesh* m, int* vertices_per_element);

/* Structured N_x x N_y quad grid on [x0,x1]x[y0,y1], each quad split along its
 * (i,j)-(i+1,j+1) diagonal into two counter-clockwise triangles, boundary tags
 * Bottom=2 Right=3 Top=4 Left=5 (src/utils/mesh_creation.cpp:249-260).  With periodic!=0
 * it also calls set_periodic("Left","Right") and set_periodic("Bottom","Top").
 * Replaces MeshSetup::create_standard_mesh (include/dgfem/utils/example_helpers.hpp:75-102)
 * for rectangles, without GMSH. */
int dgx_mesh_create_rectangle(int nx, int ny, double x0, double x1, double y0, double y1,
                              int periodic, dgx_mesh** out);

/* The same grid with the N_x x N_y cells themselves as counter-clockwise bilinear
 * quadrilaterals (vertex ids (i,j), (i+1,j), (i+1,j+1), (i,j+1)); replaces
 * MeshCreator::create_rectangular_mesh(dx, use_triangles = false, ...)
 * (include/dgfem/utils/mesh_creation.hpp:36-38) without GMSH. */
int dgx_mesh_create_rectangle_quad(int nx, int ny, double x0, double x1, double y0, double y1,
                                   int periodic, dgx_mesh** out);

/* DGMesh::set_periodic_boundaries, include/dgfem/core/mesh.hpp:102, src/core/mesh.cpp:482-588 */
int dgx_mesh_set_periodic(dgx_mesh* m, const char* tag1, const char* tag2);

/* DGMesh::set_boundary_condition_euler with a constant BoundaryConditionEuler,
 * include/dgfem/core/mesh.hpp:84-85.  value: conserved state (FAR_FIELD) or primitive
 * state (NO_SLIP_WALL); ignored for SLIP_WALL.  Must precede dgx_create. */
int dgx_mesh_set_bc(dgx_mesh* m, const char* tag, int bc_type, const double* value4);

/* counts: elements, interior faces (DGMesh::get_interior_faces), boundary faces */
int dgx_mesh_info(const dgx_mesh* m, int* n_elements, int* n_interior_faces, int* n_boundary_faces);
/* FaceConnectivity list (include/dgfem/core/mesh.hpp:147-157): [n][5] = (elem_L, elem_R,
 * face_L, face_R, reversed) in DGMesh::build_precomputed_faces order. */
int dgx_mesh_interior_faces(const dgx_mesh* m, int* out5);
/* [n][3] = (elem, face, tag id) of boundary faces, in build_precomputed_faces order */
int dgx_mesh_boundary_faces(const dgx_mesh* m, int* out3);
/* vertices [n_vertices][2] / elements [n_elements][vertices per element]; either
 * pointer may be NULL */
int dgx_mesh_arrays(const dgx_mesh* m, int* n_vertices, double* vertices, int* elements);
void dgx_mesh_destroy(dgx_mesh* m);

/* ---------------------------------------------------------------- context */

/* Builds the device-resident solver: DGMesh::initialize_dg_space (src/core/mesh.cpp:53-99),
 * DGAssembler(mesh, weak_form) (include/dgfem/solver/assembler.hpp:30-31) and
 * CompressibleDGSolverBase::compute_mass_matrix_inverse_blocks
 * (src/solver/compressible_solver_base.cpp:41-52).  The context owns all device memory. */
int dgx_create(const dgx_mesh* m, const dgx_params* params, dgx_ctx** out);
void dgx_destroy(dgx_ctx* c);
/* sizes: n_elements, n_basis (Np), n_quad (volume points), n_face_quad */
int dgx_info(const dgx_ctx* c, int* n_elements, int* n_basis, int* n_quad, int* n_face_quad);

/* ---------------------------------------------------------------- hot path (device) */

/* DGAssembler::assemble_euler_residual(u_coeffs, residuals_out),
 * include/dgfem/solver/assembler.hpp:58-59, src/solver/assembler.cpp:137-279.
 * u, r: device states.  r may not alias u. */
int dgx_residual(dgx_ctx* c, const double* u, double* r, void* stream);

/* CompressibleDGSolverBase::apply_mass_inv, include/dgfem/solver/dg_solver.hpp:236,
 * src/solver/compressible_solver_base.cpp:54-61 (also BlockMassMatrix::apply_inverse,
 * include/dgfem/solver/time_stepping.hpp:114).  in may alias out. */
int dgx_apply_mass_inv(dgx_ctx* c, const double* in, double* out, void* stream);

/* rhs_func = apply_mass_inv(assemble_residual(u)), src/solver/compressible_solver_base.cpp:108-110 */
int dgx_rhs(dgx_ctx* c, const double* u, double* du, void* stream);

/* CompressibleDGSolverBase::time_step_ssp_rk3 + SSP_RK::step_rk3,
 * include/dgfem/solver/dg_solver.hpp:239, include/dgfem/solver/time_stepping.hpp:39-55.
 * Advances u (device, in place) by n_steps SSP-RK3 steps of size dt.  The three stages
 * of a step are captured once into a CUDA graph and replayed.  Mixed precision: the stage
 * residuals and increments are FP32; u is read by the first step and written by the last,
 * and between the steps of one call the state is a double-float pair (an FP32 value and
 * its FP32 remainder, 48 significant bits) updated with exact FP32 sums, so no step but
 * the first and the last uses the FP64 pipe (a call of one step adds in FP64). */
int dgx_rk3_step(dgx_ctx* c, double* u, double dt, int n_steps, void* stream);

/* One stage of time_step_ssp_rk3 (include/dgfem/solver/time_stepping.hpp:39-55) on device
 * states, for drivers that exchange data between stages (element partitions with a halo
 * exchange): stage 1: out = u_s + dt L(u_s) (u_s = u_n); stage 2: out = 3/4 u_n + 1/4 (u_s +
 * dt L(u_s)); stage 3: out = 1/3 u_n + 2/3 (u_s + dt L(u_s)), L = M^-1 R.  Each stage is the
 * launch dgx_rk3_step makes for it, so three calls equal one step bit for bit.  FP64 and
 * double-float contexts; out may alias u_n but not u_s. */
int dgx_rk3_stage(dgx_ctx* c, const double* u_n, const double* u_s, double* out, double dt, int stage,
                  void* stream);

/* CompressibleDGSolverBase::compute_max_cfl / compute_density_range,
 * src/solver/compressible_solver_base.cpp:114-199.  Results are written to host memory
 * (the call synchronises the stream).  CFL is +inf when rho<=0 or p<=0 anywhere. */
int dgx_max_cfl(dgx_ctx* c, const double* u, double dt, double* cfl, void* stream);
int dgx_density_range(dgx_ctx* c, const double* u, double* rho_min, double* rho_max, void* stream);
/* 1 if any entry of u is NaN (the per-step scan of run_time_integration,
 * src/solver/compressible_solver_base.cpp:290-301), else 0; host result, synchronises. */
int dgx_has_nan(dgx_ctx* c, const double* u, int* has_nan, void* stream);

/* Failure detection: whether an SSP-RK3 step on this context (dgx_rk3_step, the host and
 * allocation-free variants) produced a NaN or Inf since the last call.  The stage kernels set
 * a device flag as they write u^{n+1}; this call reads and clears it (synchronising with
 * `stream`).  Returns DGX_ERR_NONFINITE with *nonfinite = 1, or DGX_OK with 0.  dgfem scans
 * the state after each step and stops the run (compressible_solver_base.cpp:290-301).
 * Returns DGX_ERR_TIMEOUT when a bounded wait inside a stage kernel (tensor-core or pipelined trace form) gave up
 * (its results are then not valid; the kernel returned and the context stays usable). */
int dgx_step_status(dgx_ctx* c, int* nonfinite, void* stream);

/* Physical coordinates of every volume quadrature point, [n_elements][n_quad][2] (host),
 * GeometricMapping::map_to_physical at the points project_initial_condition uses. */
int dgx_quad_points(const dgx_ctx* c, double* xq);
/* The same points written to device memory xq (n_elements * n_quad * 2 doubles), stream-ordered,
 * for evaluating an initial condition on the GPU before dgx_project. */
int dgx_quad_points_device(const dgx_ctx* c, double* xq, void* stream);
/* CompressibleDGSolverBase::project_initial_condition, src/solver/compressible_solver_base.cpp:63-104:
 * uq = the initial condition at dgx_quad_points, [n_elements][n_quad][4] (device). */
int dgx_project(dgx_ctx* c, const double* uq, double* u, void* stream);

/* ---------------------------------------------------------------- device states for callers without CUDA */
/* A device buffer for one state of this context (n_elements * n_basis * 4 doubles) on the
 * context's device, for callers that do not link the CUDA runtime themselves (the C++ layer's
 * solve() keeps its state there between steps).  Free it with dgx_state_free. */
int dgx_state_alloc(const dgx_ctx* c, double** u);
void dgx_state_free(double* u);
/* Copies one state: to_device != 0: host src -> device dst, else device src -> host dst.
 * Synchronous. */
int dgx_state_copy(const dgx_ctx* c, double* dst, const double* src, int to_device);

/* ---------------------------------------------------------------- host-pointer variants */
/* Synchronous: each first waits for all work on the device (calls made earlier on any
 * stream), then copies in, computes and copies out on the context's own streams. */

/* assemble_euler_residual on host states (copies in, computes, copies out). */
int dgx_residual_host(dgx_ctx* c, const double* u, double* r);
/* time_step_ssp_rk3 on a host state, in place (copies in, n_steps steps, copies out; in
 * mixed precision on triangles the copy back overlaps the last stage, range by range). */
int dgx_rk3_step_host(dgx_ctx* c, double* u, double dt, int n_steps);
/* apply_mass_inv on host states (copies in, computes, copies out). */
int dgx_apply_mass_inv_host(dgx_ctx* c, const double* in, double* out);
/* project_initial_condition on host arrays: uq [n_elements][n_quad][4] (the initial condition
 * at dgx_quad_points), u the projected state. */
int dgx_project_host(dgx_ctx* c, const double* uq, double* u);
/* compute_max_cfl, compute_density_range and the NaN scan of run_time_integration on a host
 * state; any output pointer may be NULL. */
int dgx_monitor_host(dgx_ctx* c, const double* u, double dt, double* cfl, double* rho_min,
                     double* rho_max, int* has_nan);

/* ---------------------------------------------------------------- differentiation (FP64 contexts) */

/* Tangent of assemble_euler_residual: dr = (dR/du) du.  Dual-number evaluation of the same
 * residual code, Euler and Navier-Stokes.  No counterpart in dgfem (it has no derivatives). */
int dgx_residual_jvp(dgx_ctx* c, const double* u, const double* du, double* dr, void* stream);
/* Adjoint of assemble_euler_residual: ubar = (dR/du)^T rbar.  Euler only; contexts with
 * slip-wall faces are rejected.  No counterpart in dgfem. */
int dgx_residual_vjp(dgx_ctx* c, const double* u, const double* rbar, double* ubar, void* stream);
/* Tangent-linear SSP-RK3 (time_stepping.hpp:39-55): advances the state u and its tangent
 * du together by n_steps steps, in place. */
int dgx_rk3_step_tlm(dgx_ctx* c, double* u, double* du, double dt, int n_steps, void* stream);
/* Adjoint of one SSP-RK3 step at u_n: ubar (the cotangent of u^{n+1}) is replaced by the
 * cotangent of u_n.  Recomputes the two intermediate stages.  Euler only. */
int dgx_rk3_step_adjoint(dgx_ctx* c, const double* u_n, double* ubar, double dt, void* stream);
/* J = sum_e sum_q w_q |J_e| ((rho u)^2 + (rho v)^2) / (2 rho) over the volume points, written to
 * host memory (synchronises) when J != NULL; its gradient dJ/du into the device state grad
 * when grad != NULL. */
int dgx_kinetic_energy(dgx_ctx* c, const double* u, double* J, double* grad, void* stream);
/* dJ/du0 for J(u(T)), u(T) = n_steps SSP-RK3 steps of size dt from u0: forward sweep with a
 * checkpoint every checkpoint_every steps, then, per segment from the last, a recomputation
 * storing each step's stages and the adjoint steps backward.  J (host, may be NULL) and
 * grad (device state) are outputs.  Allocates its checkpoint storage for the call.  Euler only. */
int dgx_kinetic_energy_gradient(dgx_ctx* c, const double* u0, double dt, int n_steps, int checkpoint_every,
                                double* J, double* grad, void* stream);
/* The same gradient with binomial checkpointing (the schedules of Griewank's revolve, found by
 * dynamic programming): n_snapshots device states beside u0 and one work state, and the fewest
 * recomputed forward steps any schedule with that memory needs: with c = n_snapshots + 1
 * checkpoints (u0 included), t n - C(c + t, t - 1) for C(c + t - 1, t - 1) < n <= C(c + t, t)
 * (Griewank and Walther, ACM TOMS 26 (2000)).  The gradient equals
 * dgx_kinetic_energy_gradient's bit for bit.
 * stats (may be NULL): [0] forward steps recomputed in the reverse sweep, [1] states held
 * (snapshots + the work state), [2] the schedule's optimum.  Rejects n_steps^2 (n_snapshots + 1)
 * > 4e9 (the schedule's host cost).  Euler only; no counterpart in dgfem. */
int dgx_kinetic_energy_gradient_binomial(dgx_ctx* c, const double* u0, double dt, int n_steps, int n_snapshots,
                                         double* J, double* grad, long long* stats, void* stream);

/* ---------------------------------------------------------------- allocation-free stepping */

/* No counterpart in dgfem.  For callers that may not allocate device memory while they
 * run (a host framework that owns all device memory through its own pool, or a loop that
 * must never enter the CUDA allocator): the same SSP-RK3 steps as dgx_rk3_step on the
 * device state u (in place), with the stage buffers taken from one static device array
 * of the library instead of memory the library allocates.  The call allocates nothing.
 *  - Limit: n_elements * n_basis * 4 <= DGX_STATIC_MAX_STATE; larger states are rejected
 *    with DGX_ERR_INVALID.  The array (5 * DGX_STATIC_MAX_STATE floats, 20 MiB) is
 *    reserved on a device when the first triangle-mesh context is created there
 *    (dgx_create loads it, looks up its device address and loads the kernels this call
 *    launches, with that device current), and it stays reserved until the process exits.
 *    Create the context before any stream capture.
 *  - All calls share the array; calls whose GPU work overlaps (other streams or threads)
 *    race on it.  Nothing in it needs to start at zero.
 *  - Mixed precision runs the stage kernel that reads neighbour coefficient rows, at one CTA
 *    per 128-element tile, not the form the autotuner picks for dgx_rk3_step (the face-trace
 *    form needs trace buffers): the results are the same bit for bit.  That kernel's stage
 *    took 187 us against 132 us for the autotuner's pick on a 524,288-element mesh (stage 2,
 *    p = 3, through dgx_rk3_step).
 *  - The context's device must be current.  Kernels are launched directly on `stream`. */
#define DGX_STATIC_MAX_STATE (1 << 20)
int dgx_rk3_step_static(dgx_ctx* c, double* u, double dt, int n_steps, void* stream);

/* ---------------------------------------------------------------- output */

/* The solution at reference points of every element, for visualisation: out (device,
 * n_elements * n_points * 4 doubles) = sum_i phi_i(ref_xy[k]) u[e][i][:], ref_xy (host,
 * n_points (xi, eta) pairs on the reference triangle (0,0),(1,0),(0,1)), at most 128 points.
 * Replaces the per-point basis evaluation of VTKWriter::evaluate_at_points
 * (src/utils/vtk_writer.cpp:285-323). */
int dgx_eval_points(dgx_ctx* c, int n_points, const double* ref_xy, const double* u, double* out, void* stream);

/* ---------------------------------------------------------------- launch shape */

/* The stage kernel the autotuner picked for a mixed-precision context: its grid (CTAs;
 * each walks the 128-element tiles with a grid stride), the number of tiles, and its form:
 * 0 = CUDA cores, neighbour coefficient rows read per face; 2 = CUDA cores, face traces
 * exchanged through HBM (Euler); 3 = the same with each CTA bulk-copying its next tile's
 * inputs while it computes a tile (Euler, meshes whose boundary faces all have a condition;
 * 2 or 3 CTAs per SM); 1 = the 3xTF32 tcgen05 tensor-core form (Euler, orders 1-3, the same
 * meshes; one CTA per SM).  grid is 0 until the first dgx_rk3_step, which times the
 * candidates on its stream: the CUDA-core forms at one CTA per tile and at 1..8 CTAs per SM,
 * and the others at their grids.  Environment: DGX_STAGE_KERNEL=rows, =trace (forms 2 and 3),
 * =pipe or =tc keeps one form; DGX_AUTOTUNE=0 skips the timing (the first candidate).
 * Quadrilateral meshes have one form (grid = tiles).  A mixed-precision state passed to
 * dgx_rk3_step must be 16-byte aligned.  No counterpart in dgfem. */
int dgx_launch_shape(const dgx_ctx* c, int* grid, int* tiles, int* form);
/* Elements per CTA of the mixed stage kernel the autotuner picked: 128, or 64 or 32 for the
 * face-trace form at smaller tiles (form 2, one CTA per tile; DGX_STAGE_KERNEL=trace64 or
 * =trace32 keeps one of those); 0 until the first dgx_rk3_step.  nbr_shared (may be NULL) is
 * 1 when that kernel copies each element's neighbour trace blocks into shared memory during
 * staging (32-element tiles, meshes whose faces are all interior or ghost faces;
 * DGX_STAGE_KERNEL=trace32s), else 0.  No counterpart in dgfem. */
int dgx_stage_tile(const dgx_ctx* c, int* elements, int* nbr_shared);

/* ---------------------------------------------------------------- batched solves */

/* No counterpart in dgfem, where an ensemble is a loop over solver objects.  n_inst
 * independent mixed-precision Euler or Navier-Stokes solves on triangle meshes, each on its
 * own mesh and order (1..4, params[i].order), advanced together: every SSP-RK3 stage of
 * every instance is one persistent kernel launch, and dgx_batch_rk3_step replays CUDA graphs
 * of those launches.  All instances share the basis, gamma and physics, and Navier-Stokes
 * instances mu, Prandtl and sigma0 (params[0]); anything else, and other precisions, are
 * rejected with DGX_ERR_INVALID.  Meshes are read at creation only. */
typedef struct dgx_batch dgx_batch;
int dgx_batch_create(int n_inst, const dgx_mesh* const* meshes, const dgx_params* params, dgx_batch** out);
void dgx_batch_destroy(dgx_batch* b);
/* Instance inst: element count, basis size and the device address of its FP64 state
 * (n_elements * n_basis * 4 doubles, dgx_residual's layout).  The batch owns the state
 * (zero after creation); callers write initial states there and read results back. */
int dgx_batch_info(const dgx_batch* b, int inst, int* n_elements, int* n_basis, double** u);
/* n_steps SSP-RK3 steps of every instance; dt: n_inst host doubles, > 0, instance i's
 * step.  The first call times the launch shapes (see dgx_launch_shape) and captures the
 * graphs; stream-ordered on `stream` after that. */
int dgx_batch_rk3_step(dgx_batch* b, const double* dt, int n_steps, void* stream);
/* The batched kernel's grid (0 until the first step) and its total number of tiles. */
int dgx_batch_launch_shape(const dgx_batch* b, int* grid, int* tiles);
/* The form the autotuner picked for a batch's stages (0 until the first step): 1 = the batched
 * kernel (one launch per stage over every order's tiles, neighbour coefficient rows); 2 = the
 * face-trace kernel of dgx_rk3_step (32-element tiles, neighbour blocks in shared memory), one
 * launch per order and stage, offered for Euler batches whose boundary faces all have a condition
 * (ghost blocks, as for a single context; DGX_STAGE_KERNEL=rows or =trace32s keeps one).  No
 * counterpart in dgfem. */
int dgx_batch_stage_form(const dgx_batch* b, int* form);

#ifdef __cplusplus
}
#endif
#endif
