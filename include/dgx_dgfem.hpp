// dgx_dgfem.hpp -- header-only C++17 layer over include/dgx.h with dgfem's class and
// method names, so dgfem (GaleAxiom/Discontinuous-Galerkin-FEM) can route its explicit
// Euler / Navier-Stokes path to the GPU without changing its callers.
//
// Mirrors (paths inside the dgfem project):
//   Mesh                         DGMesh, include/dgfem/core/mesh.hpp:29-228
//   EulerWeakFormulation         include/dgfem/weak_forms/euler_weak_formulation.hpp:16-132
//   NavierStokesWeakFormulation  include/dgfem/weak_forms/navier_stokes_weak_formulation.hpp:17-80
//   Assembler                    DGAssembler::assemble_euler_residual, include/dgfem/solver/assembler.hpp:58-59
//   EulerDGSolver, NavierStokesDGSolver
//                                include/dgfem/solver/dg_solver.hpp:223-296 (apply_mass_inv,
//                                time_step_ssp_rk3, compute_max_cfl, compute_density_range)
//
// Matrices: any MatrixT with rows(), cols(), operator()(i, j) and resize(r, c) -- dgfem's
// Eigen::MatrixXd, or a stand-in.  A state is std::vector<MatrixT> of Np x 4 blocks, as in
// dgfem; conversion to the C ABI's flat layout (elem*Np*4 + i*4 + v) happens here.
// Errors: DGX_ERR_INVALID -> std::invalid_argument, DGX_ERR_RANGE -> std::out_of_range,
// anything else -> std::runtime_error, each with dgx_last_error()'s message.
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "dgx.h"

namespace dgx_dgfem {

inline void check(int rc) {
    if (rc == DGX_OK) return;
    const std::string msg = dgx_last_error();
    if (rc == DGX_ERR_INVALID) throw std::invalid_argument(msg);
    if (rc == DGX_ERR_RANGE) throw std::out_of_range(msg);
    throw std::runtime_error(msg);
}

// DGMesh(vertices, elements, element_tags, boundary_tags, boundary_edges).  VertMat: n x 2,
// ElemMat: n x 3 triangles or n x 4 quadrilaterals (Eigen::MatrixXd / MatrixXi or anything
// with rows(), cols() and operator()); the column count picks the element type as in
// DGMesh's constructor (src/core/mesh.cpp:23-35).
class Mesh {
public:
    template <class VertMat, class ElemMat>
    Mesh(const VertMat& vertices, const ElemMat& elements,
         const std::map<std::string, int>& boundary_tags,
         const std::map<int, std::vector<std::pair<int, int>>>& boundary_edges) {
        std::vector<double> v((size_t)vertices.rows() * 2);
        for (long i = 0; i < (long)vertices.rows(); ++i) {
            v[2 * i] = vertices(i, 0);
            v[2 * i + 1] = vertices(i, 1);
        }
        const int nvpe = (int)elements.cols();
        std::vector<int> e((size_t)elements.rows() * (nvpe > 0 ? nvpe : 1));
        for (long i = 0; i < (long)elements.rows(); ++i)
            for (int k = 0; k < nvpe; ++k) e[(size_t)nvpe * i + k] = (int)elements(i, k);
        std::vector<const char*> names;
        std::vector<int> ids;
        for (const auto& t : boundary_tags) {
            names.push_back(t.first.c_str());
            ids.push_back(t.second);
        }
        std::vector<int> b;
        for (const auto& te : boundary_edges)  // std::map: tags in ascending order, as dgfem
            for (const auto& ed : te.second) {
                b.push_back(te.first);
                b.push_back(ed.first);
                b.push_back(ed.second);
            }
        check(dgx_mesh_create_nv(nvpe, (int)vertices.rows(), v.data(), (int)elements.rows(), e.data(),
                                 (int)names.size(), names.data(), ids.data(), (int)b.size() / 3, b.data(), &m_));
    }
    Mesh(const Mesh&) = delete;
    Mesh& operator=(const Mesh&) = delete;
    ~Mesh() { dgx_mesh_destroy(m_); }

    void set_periodic_boundaries(const std::string& t1, const std::string& t2) {
        check(dgx_mesh_set_periodic(m_, t1.c_str(), t2.c_str()));
    }
    // constant BoundaryConditionEuler (FAR_FIELD: conserved state; NO_SLIP_WALL: primitive)
    void set_boundary_condition_euler(const std::string& tag, int bc_type, const double value[4]) {
        check(dgx_mesh_set_bc(m_, tag.c_str(), bc_type, value));
    }
    // "triangle" or "quad" (DGMesh::get_element_type)
    std::string get_element_type() const {
        int nvpe = 3;
        check(dgx_mesh_vertices_per_element(m_, &nvpe));
        return nvpe == 4 ? "quad" : "triangle";
    }
    int get_n_elements() const {
        int ne = 0;
        check(dgx_mesh_info(m_, &ne, nullptr, nullptr));
        return ne;
    }
    dgx_mesh* handle() const { return m_; }

private:
    dgx_mesh* m_ = nullptr;
};

struct EulerWeakFormulation {
    explicit EulerWeakFormulation(double gamma = 1.4) : gamma_(gamma) {}
    double get_gamma() const { return gamma_; }
    virtual bool has_viscous_terms() const { return false; }
    virtual ~EulerWeakFormulation() = default;
    virtual void fill(dgx_params& p) const {
        p.physics = DGX_EULER;
        p.gamma = gamma_;
    }

protected:
    double gamma_;
};

struct NavierStokesWeakFormulation : EulerWeakFormulation {
    NavierStokesWeakFormulation(double gamma = 1.4, double dynamic_viscosity = 1.0e-3, double prandtl = 0.72,
                                double penalty_prefactor = 5.0)
        : EulerWeakFormulation(gamma), mu_(dynamic_viscosity), pr_(prandtl), s0_(penalty_prefactor) {
        if (mu_ <= 0.0) throw std::invalid_argument("Dynamic viscosity must be positive for Navier-Stokes weak formulation");
        if (pr_ <= 0.0) throw std::invalid_argument("Prandtl number must be positive for Navier-Stokes weak formulation");
        if (s0_ <= 0.0) throw std::invalid_argument("Penalty prefactor must be positive for Navier-Stokes weak formulation");
    }
    bool has_viscous_terms() const override { return true; }
    double compute_penalty_parameter(int p, double h) const {
        return s0_ * mu_ * (p + 1) * (p + 1) / (h > 1e-12 ? h : 1e-12);
    }
    void fill(dgx_params& p) const override {
        p.physics = DGX_NAVIER_STOKES;
        p.gamma = gamma_;
        p.mu = mu_;
        p.prandtl = pr_;
        p.sigma0 = s0_;
    }

private:
    double mu_, pr_, s0_;
};

// DGAssembler + the compressible solvers' protected hot-path methods, on the GPU.
class Assembler {
public:
    Assembler(const Mesh& mesh, int order, int basis, const EulerWeakFormulation& wf, int precision = DGX_FP64) {
        dgx_params p{};
        p.order = order;
        p.basis = basis;
        p.precision = precision;
        wf.fill(p);
        check(dgx_create(mesh.handle(), &p, &c_));
        check(dgx_info(c_, &ne_, &np_, nullptr, nullptr));
    }
    Assembler(const Assembler&) = delete;
    Assembler& operator=(const Assembler&) = delete;
    ~Assembler() { dgx_destroy(c_); }

    int n_elements() const { return ne_; }
    int n_basis() const { return np_; }
    dgx_ctx* handle() const { return c_; }

    // DGAssembler::assemble_euler_residual: residuals_out is resized and overwritten.
    template <class MatrixT>
    void assemble_euler_residual(const std::vector<MatrixT>& u_coeffs, std::vector<MatrixT>& residuals_out) {
        std::vector<double> u = flatten(u_coeffs), r(u.size());
        check(dgx_residual_host(c_, u.data(), r.data()));
        unflatten(r, residuals_out);
    }

    // CompressibleDGSolverBase::apply_mass_inv
    template <class MatrixT>
    std::vector<MatrixT> apply_mass_inv(const std::vector<MatrixT>& vec) {
        std::vector<double> a = flatten(vec), b(a.size());
        check(dgx_apply_mass_inv_host(c_, a.data(), b.data()));
        std::vector<MatrixT> out;
        unflatten(b, out);
        return out;
    }

    // CompressibleDGSolverBase::time_step_ssp_rk3
    template <class MatrixT>
    std::vector<MatrixT> time_step_ssp_rk3(const std::vector<MatrixT>& u_n, double dt) {
        std::vector<double> u = flatten(u_n);
        check(dgx_rk3_step_host(c_, u.data(), dt, 1));
        std::vector<MatrixT> out;
        unflatten(u, out);
        return out;
    }

    // CompressibleDGSolverBase::compute_max_cfl / compute_density_range
    template <class MatrixT>
    double compute_max_cfl(const std::vector<MatrixT>& u, double dt) {
        std::vector<double> f = flatten(u);
        double cfl = 0.0;
        check(dgx_monitor_host(c_, f.data(), dt, &cfl, nullptr, nullptr, nullptr));
        return cfl;
    }
    template <class MatrixT>
    std::pair<double, double> compute_density_range(const std::vector<MatrixT>& u) {
        std::vector<double> f = flatten(u);
        double lo = 0.0, hi = 0.0;
        check(dgx_monitor_host(c_, f.data(), 0.0, nullptr, &lo, &hi, nullptr));
        return {lo, hi};
    }

private:
    template <class MatrixT>
    std::vector<double> flatten(const std::vector<MatrixT>& u) const {
        if ((int)u.size() != ne_) throw std::invalid_argument("state has the wrong number of elements");
        std::vector<double> f((size_t)ne_ * np_ * 4);
        for (int e = 0; e < ne_; ++e) {
            if ((int)u[e].rows() != np_ || (int)u[e].cols() != 4)
                throw std::invalid_argument("element block must be n_basis x 4");
            for (int i = 0; i < np_; ++i)
                for (int v = 0; v < 4; ++v) f[((size_t)e * np_ + i) * 4 + v] = u[e](i, v);
        }
        return f;
    }
    template <class MatrixT>
    void unflatten(const std::vector<double>& f, std::vector<MatrixT>& u) const {
        u.resize(ne_);
        for (int e = 0; e < ne_; ++e) {
            if ((int)u[e].rows() != np_ || (int)u[e].cols() != 4) u[e].resize(np_, 4);
            for (int i = 0; i < np_; ++i)
                for (int v = 0; v < 4; ++v) u[e](i, v) = f[((size_t)e * np_ + i) * 4 + v];
        }
    }

    dgx_ctx* c_ = nullptr;
    int ne_ = 0, np_ = 0;
};

// EulerDGSolver(mesh, gamma) / NavierStokesDGSolver(mesh, gamma, mu, Pr, sigma0): the
// hot-path methods of CompressibleDGSolverBase over an Assembler.
class EulerDGSolver : public Assembler {
public:
    EulerDGSolver(const Mesh& mesh, int order, int basis, double gamma = 1.4, int precision = DGX_FP64)
        : Assembler(mesh, order, basis, EulerWeakFormulation(gamma), precision) {}
};

class NavierStokesDGSolver : public Assembler {
public:
    NavierStokesDGSolver(const Mesh& mesh, int order, int basis, double gamma = 1.4, double mu = 1.0e-3,
                         double prandtl = 0.72, double sigma0 = 5.0, int precision = DGX_FP64)
        : Assembler(mesh, order, basis, NavierStokesWeakFormulation(gamma, mu, prandtl, sigma0), precision) {}
};

}  // namespace dgx_dgfem
