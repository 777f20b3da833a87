/*
 * dg_oracle.h -- CPU restatement of dgfem's explicit DG residual-and-update path.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the parity checker for the GPU path and
 * the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs may load it; the GPU product never links or calls it.
 *
 * What it restates (paths inside the dgfem project):
 *   quadrature   src/quadrature/factory.cpp:75-236, 238-717 (tables generated from it)
 *   bases        src/basis/monomial.cpp:30-72, src/basis/dubiner.cpp:24-168
 *   mapping      src/reference/mapping.cpp:22-58, src/reference/elements.cpp:27-61
 *   space        src/core/space.cpp:20-67, 69-288
 *   mesh         src/core/mesh.cpp:18-51, 312-480, 482-588
 *   Euler form   src/weak_forms/euler_weak_formulation.cpp:27-296
 *   NS form      src/weak_forms/navier_stokes_weak_formulation.cpp:36-278
 *   assembler    src/solver/assembler.cpp:137-279
 *   mass / RK3   src/weak_forms/weak_formulation_base.cpp:198-217,
 *                src/solver/compressible_solver_base.cpp:41-170,
 *                include/dgfem/solver/time_stepping.hpp:39-85
 *
 * Pinning: dgfem cannot be compiled here (Eigen, GMSH and GoogleTest are absent), so
 * the oracle is pinned by re-running dgfem's own known-answer tests against it
 * (quadrature exactness, basis values/Gram/gradients, mapping, face integrals, the
 * Navier-Stokes viscous residual KATs on the two-triangle mesh).  The inviscid Euler
 * residual, Rusanov flux, mass inverse and RK3 have no known-answer test in dgfem;
 * for those the oracle is checked by property tests (free-stream preservation,
 * Rusanov antisymmetry, discrete conservation, exact-vortex convergence).
 *
 * Arithmetic: FP64, built without fast-math and with FMA contraction off so results
 * are identical on x86-64 and aarch64 hosts.
 *
 * Layout: a state is double[n_elem][n_basis][4] -- dgfem's flat DGSolution index
 * elem*Np*V + i*V + v (src/core/solution.cpp:143-145).
 */
#ifndef DG_ORACLE_H
#define DG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BASIS_MONOMIAL = 0, ORC_BASIS_DUBINER = 1, ORC_BASIS_LEGENDRE = 2 /* quads */ };
enum { ORC_BC_FAR_FIELD = 0, ORC_BC_SLIP_WALL = 1, ORC_BC_NO_SLIP_WALL = 2, ORC_BC_PERIODIC = 3 };

typedef void (*orc_bc_fn)(double x, double y, double* out4, void* user);
typedef struct orc_mesh orc_mesh;

/* quadrature and bases */
int orc_tri_rule(int order, int* n, const double** pts, const double** wts);
int orc_gl_rule(int n, const double** pts, const double** wts);
int orc_n_basis(int p);
void orc_basis_eval(int basis, int p, double x, double y, double* phi);
void orc_basis_grad(int basis, int p, double x, double y, double* grad /* [np][2] */);
/* nv = 3 (P1 triangle on (0,0),(1,0),(0,1)) or 4 (bilinear quad on [-1,1]^2) */
int orc_compute_mapping_nv(int nv, const double* verts, double xi, double eta, double* xp, double* J_det,
                           double* dxi_dx);
void orc_map_face_point_nv(int nv, int face, double s, double* xi);
int orc_compute_mapping(const double* verts /* [3][2] */, double xi, double eta,
                        double* x_phys /* [2] */, double* J_det, double* dxi_dx /* [2][2] */);
void orc_map_face_point(int face, double s, double* xi /* [2] */);

/* mesh: DGMesh(vertices, elements, tags, boundary_tags, boundary_edges) */
/* nvpe = 3 (triangles) or 4 (quads: elements [n][4], counter-clockwise) */
orc_mesh* orc_mesh_create_nv(int nvpe, int nv, const double* verts, int ne, const int* elems, int n_bedge,
                             const int* bedges);
int orc_mesh_nvpe(const orc_mesh* m);
orc_mesh* orc_mesh_create(int n_vert, const double* vertices, int n_elem, const int* elements,
                          int n_bedge, const int* bedges /* [n][3]: tag, v1, v2 (tag-sorted) */);
void orc_mesh_destroy(orc_mesh* m);
int orc_mesh_set_periodic(orc_mesh* m, int tag1, int tag2, int match_on_y);
int orc_mesh_init_space(orc_mesh* m, int order, int basis);
int orc_mesh_rebuild_faces(orc_mesh* m);
int orc_mesh_n_interior_faces(const orc_mesh* m);
int orc_mesh_n_boundary_faces(const orc_mesh* m);
void orc_mesh_interior_faces(const orc_mesh* m, int* out /* [n][5]: L, R, fL, fR, reversed */);
void orc_mesh_boundary_faces(const orc_mesh* m, int* out /* [n][3]: elem, face, tag */);
void orc_mesh_neighbors(const orc_mesh* m, int* out /* [ne][3][2] */);
int orc_mesh_set_bc(orc_mesh* m, int tag, int type, const double* value4, orc_bc_fn fn, void* user);
void orc_mesh_space_dims(const orc_mesh* m, int* np, int* nq, int* nfq);
/* element/face data exactly as DGSpace stores it */
void orc_mesh_element_data(const orc_mesh* m, int e, double* J_det /* [nq] */,
                           double* dphi_dx /* [nq*np][2] */);
void orc_mesh_face_data(const orc_mesh* m, int e, int f, double* normal /* [2] */,
                        double* length, double* quad_points /* [2*nfq] col-major */,
                        double* dphi_dx_face /* [nfq*np][2] */);
void orc_space_tables(const orc_mesh* m, double* phi_vol /* [nq][np] */,
                      double* phi_face /* [3][nfq][np] */, double* vol_w, double* face_w);
void orc_mesh_quad_points(const orc_mesh* m, double* xq /* [ne][nq][2] */);

/* physics */
typedef struct {
    double gamma;
    int viscous;      /* 0: EulerWeakFormulation, 1: NavierStokesWeakFormulation */
    double mu, prandtl, sigma0;
} orc_physics;

void orc_set_threads(int n);
void orc_rusanov(double gamma, const double* UL, const double* UR, const double* n, double* H);
void orc_viscous_flux(const orc_physics* ph, const double* U, const double* gradU /* [4][2] */,
                      double* Fv, double* Gv);
double orc_penalty(const orc_physics* ph, int p, double h);
int orc_volume_residual(const orc_mesh* m, const orc_physics* ph, int e, const double* u, double* R);
int orc_viscous_volume_residual(const orc_mesh* m, const orc_physics* ph, int e, const double* u,
                                double* R);
int orc_interior_face_residual(const orc_mesh* m, const orc_physics* ph, int k, const double* u,
                               int viscous, double* RL, double* RR);
int orc_boundary_face_residual(const orc_mesh* m, const orc_physics* ph, int k, const double* u,
                               int viscous, double* R);
int orc_assemble_residual(const orc_mesh* m, const orc_physics* ph, const double* u, double* R);
int orc_mass_matrix(const orc_mesh* m, int e, double* M /* [np][np] */);
int orc_compute_mass_inverse(orc_mesh* m);
int orc_apply_mass_inv(const orc_mesh* m, const double* in, double* out);
int orc_rhs(const orc_mesh* m, const orc_physics* ph, const double* u, double* du);
int orc_rk3_step(const orc_mesh* m, const orc_physics* ph, double* u, double dt);
double orc_max_cfl(const orc_mesh* m, double gamma, const double* u, double dt);
void orc_density_range(const orc_mesh* m, const double* u, double* rho_min, double* rho_max);
int orc_project(const orc_mesh* m, const double* Uq /* [ne][nq][4] */, double* u);

#ifdef __cplusplus
}
#endif
#endif
