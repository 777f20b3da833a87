// dgx_dgfem.hpp -- header-only C++17 layer over include/dgx.h with dgfem's class shapes, so
// dgfem (GaleAxiom/Discontinuous-Galerkin-FEM) code that builds a mesh, a space, a weak form and
// a solver runs its explicit Euler / Navier-Stokes path on the GPU with the same calls.
//
// Mirrors (paths inside the dgfem project):
//   DGMesh                      include/dgfem/core/mesh.hpp:29-228 (constructor :31-33,
//                               initialize_dg_space :44, set_boundary_condition_euler :84-85,
//                               set_periodic_boundaries :102, get_element_type :123, get_dg_space :126)
//   DGSpace                     include/dgfem/core/space.hpp:25-27 (DGSpace(element_type, order))
//   BCTypeEuler / BoundaryConditionEuler   include/dgfem/boundary/conditions.hpp:27-103 (constant values)
//   EulerWeakFormulation        include/dgfem/weak_forms/euler_weak_formulation.hpp:16-132
//   NavierStokesWeakFormulation include/dgfem/weak_forms/navier_stokes_weak_formulation.hpp:17-80
//   DGAssembler                 include/dgfem/solver/assembler.hpp:30-31 (DGAssembler(mesh, weak_form)),
//                               :58-59 (assemble_euler_residual)
//   CompressibleDGSolverBase, EulerDGSolver, NavierStokesDGSolver
//                               include/dgfem/solver/dg_solver.hpp:223-296 (solve, time_step_ssp_rk3,
//                               apply_mass_inv, project_initial_condition, compute_max_cfl,
//                               compute_density_range)
//
// Matrix and vector types: Eigen's (MatrixXd, MatrixXi, VectorXi, Vector2d, Vector4d) when
// <Eigen/Dense> is on the include path, as inside dgfem; otherwise small stand-ins below with
// the part of Eigen's interface this layer uses.  A state is std::vector<MatrixXd> of Np x 4
// blocks, as in dgfem; the C ABI's flat layout (elem*Np*4 + i*4 + v) is converted here.
// Errors: DGX_ERR_INVALID -> std::invalid_argument, DGX_ERR_RANGE -> std::out_of_range,
// anything else -> std::runtime_error, each with dgx_last_error()'s message.
// Precision: dgfem computes in FP64 (DGX_FP64, the default here); the solver and assembler
// constructors take DGX_MIXED or DGX_DF64 as an optional last argument.
#pragma once

#include <cmath>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

#include "dgx.h"

#if __has_include(<Eigen/Dense>)
#include <Eigen/Dense>
namespace dgx_dgfem {
using MatrixXd = Eigen::MatrixXd;
using MatrixXi = Eigen::MatrixXi;
using VectorXi = Eigen::VectorXi;
using Vector2d = Eigen::Vector2d;
using Vector4d = Eigen::Vector4d;
}  // namespace dgx_dgfem
#else
namespace dgx_dgfem {
// Dense column-major matrix with the subset of Eigen's interface used by this layer.
template <class T>
class DenseMatrix {
public:
    DenseMatrix() = default;
    DenseMatrix(long r, long c) { resize(r, c); }
    long rows() const { return r_; }
    long cols() const { return c_; }
    long size() const { return r_ * c_; }
    void resize(long r, long c) {
        r_ = r;
        c_ = c;
        a_.assign((size_t)(r * c), T(0));
    }
    T& operator()(long i, long j) { return a_[(size_t)(j * r_ + i)]; }
    const T& operator()(long i, long j) const { return a_[(size_t)(j * r_ + i)]; }
    T& operator()(long i) { return a_[(size_t)i]; }
    const T& operator()(long i) const { return a_[(size_t)i]; }

private:
    long r_ = 0, c_ = 0;
    std::vector<T> a_;
};
using MatrixXd = DenseMatrix<double>;
using MatrixXi = DenseMatrix<int>;
struct VectorXi : DenseMatrix<int> {
    VectorXi() = default;
    explicit VectorXi(long n) : DenseMatrix<int>(n, 1) {}
};
template <int N>
struct FixedVector {
    double v[N] = {};
    FixedVector() = default;
    template <class... A>
    FixedVector(A... a) : v{(double)a...} {}
    double& operator()(int i) { return v[i]; }
    double operator()(int i) const { return v[i]; }
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
    double x() const { return v[0]; }
    double y() const { return v[1]; }
};
using Vector2d = FixedVector<2>;
using Vector4d = FixedVector<4>;
}  // namespace dgx_dgfem
#endif

namespace dgx_dgfem {

inline void check(int rc) {
    if (rc == DGX_OK) return;
    const std::string msg = dgx_last_error();
    if (rc == DGX_ERR_INVALID) throw std::invalid_argument(msg);
    if (rc == DGX_ERR_RANGE) throw std::out_of_range(msg);
    throw std::runtime_error(msg);
}

// BCTypeEuler and a constant BoundaryConditionEuler (conserved state for FAR_FIELD, primitive
// state for NO_SLIP_WALL, nothing for SLIP_WALL).
enum class BCTypeEuler { FAR_FIELD = DGX_BC_FAR_FIELD, SLIP_WALL = DGX_BC_SLIP_WALL,
                         NO_SLIP_WALL = DGX_BC_NO_SLIP_WALL, PERIODIC = DGX_BC_PERIODIC };

class BoundaryConditionEuler {
public:
    explicit BoundaryConditionEuler(BCTypeEuler type, const Vector4d& value = Vector4d(0.0, 0.0, 0.0, 0.0))
        : type_(type) {
        for (int v = 0; v < 4; ++v) value_[v] = value(v);
    }
    BCTypeEuler get_type() const { return type_; }
    const double* value() const { return value_; }

private:
    BCTypeEuler type_;
    double value_[4];
};

// DGSpace(element_type, order).  dgfem's triangle space uses the monomial basis and its quad
// space the Legendre basis (src/core/space.cpp:307-319); `basis` may name DGX_BASIS_DUBINER for
// triangles instead.
class DGSpace {
public:
    DGSpace(std::string_view element_type, int order, int basis = -1)
        : type_(element_type), order_(order) {
        if (type_ != "triangle" && type_ != "quad") throw std::invalid_argument("Unsupported element type: " + type_);
        basis_ = basis >= 0 ? basis : (type_ == "quad" ? DGX_BASIS_LEGENDRE : DGX_BASIS_MONOMIAL);
    }
    int get_order() const noexcept { return order_; }
    const std::string& get_element_type() const noexcept { return type_; }
    int get_basis() const noexcept { return basis_; }

private:
    std::string type_;
    int order_;
    int basis_;
};

// DGMesh(vertices, elements, element_tags, boundary_tags, boundary_edges).  VertMat: n x 2,
// ElemMat: n x 3 triangles or n x 4 quadrilaterals (the column count picks the element type, as
// in src/core/mesh.cpp:23-35), TagVec: per-element tags (unused by the explicit path).
class DGMesh {
public:
    template <class VertMat, class ElemMat, class TagVec>
    DGMesh(const VertMat& vertices, const ElemMat& elements, const TagVec& /*element_tags*/,
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
        type_ = nvpe == 4 ? "quad" : "triangle";
    }
    DGMesh(const DGMesh&) = delete;
    DGMesh& operator=(const DGMesh&) = delete;
    ~DGMesh() { dgx_mesh_destroy(m_); }

    // DGMesh::initialize_dg_space: the space the assembler and solvers build on
    void initialize_dg_space(std::shared_ptr<DGSpace> dg_space, int n_variables = 1) {
        if (!dg_space) throw std::invalid_argument("DG space must not be null");
        if (dg_space->get_element_type() != type_)
            throw std::invalid_argument("DG space element type does not match the mesh");
        space_ = std::move(dg_space);
        n_vars_ = n_variables;
    }
    void set_periodic_boundaries(std::string_view t1, std::string_view t2) {
        check(dgx_mesh_set_periodic(m_, std::string(t1).c_str(), std::string(t2).c_str()));
    }
    void set_boundary_condition_euler(std::string_view tag, std::shared_ptr<BoundaryConditionEuler> bc) {
        if (!bc) throw std::invalid_argument("boundary condition must not be null");
        check(dgx_mesh_set_bc(m_, std::string(tag).c_str(), (int)bc->get_type(), bc->value()));
    }
    const std::string& get_element_type() const noexcept { return type_; }
    std::shared_ptr<DGSpace> get_dg_space() const noexcept { return space_; }
    int get_n_elements() const {
        int ne = 0;
        check(dgx_mesh_info(m_, &ne, nullptr, nullptr));
        return ne;
    }
    dgx_mesh* handle() const noexcept { return m_; }

private:
    dgx_mesh* m_ = nullptr;
    std::string type_;
    std::shared_ptr<DGSpace> space_;
    int n_vars_ = 1;
};
using Mesh = DGMesh;

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

// DGAssembler(mesh, weak_form): the GPU context for the mesh's DG space and the weak form.
class DGAssembler {
public:
    template <typename WeakFormT>
    DGAssembler(std::shared_ptr<DGMesh> mesh, std::shared_ptr<WeakFormT> weak_form, int precision = DGX_FP64)
        : mesh_(std::move(mesh)) {
        if (!mesh_ || !weak_form) throw std::invalid_argument("DGAssembler: mesh and weak form must not be null");
        const std::shared_ptr<DGSpace> space = mesh_->get_dg_space();
        if (!space) throw std::runtime_error("DG space not initialized in mesh");
        dgx_params p{};
        p.order = space->get_order();
        p.basis = space->get_basis();
        p.precision = precision;
        static_cast<const EulerWeakFormulation&>(*weak_form).fill(p);
        check(dgx_create(mesh_->handle(), &p, &c_));
        check(dgx_info(c_, &ne_, &np_, &nq_, nullptr));
    }
    DGAssembler(const DGAssembler&) = delete;
    DGAssembler& operator=(const DGAssembler&) = delete;
    virtual ~DGAssembler() { dgx_destroy(c_); }

    int n_elements() const noexcept { return ne_; }
    int n_basis() const noexcept { return np_; }
    dgx_ctx* handle() const noexcept { return c_; }

    // DGAssembler::assemble_euler_residual: residuals_out is resized and overwritten.
    template <class MatrixT>
    void assemble_euler_residual(const std::vector<MatrixT>& u_coeffs, std::vector<MatrixT>& residuals_out) {
        std::vector<double> u = flatten(u_coeffs), r(u.size());
        check(dgx_residual_host(c_, u.data(), r.data()));
        unflatten(r, residuals_out);
    }

protected:
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

    std::shared_ptr<DGMesh> mesh_;
    dgx_ctx* c_ = nullptr;
    int ne_ = 0, np_ = 0, nq_ = 0;
};

// A state held on the context's device (RAII over dgx_state_alloc / dgx_state_free).
class DeviceState {
public:
    explicit DeviceState(const DGAssembler& a) : c_(a.handle()) { check(dgx_state_alloc(c_, &u_)); }
    DeviceState(const DeviceState&) = delete;
    DeviceState& operator=(const DeviceState&) = delete;
    ~DeviceState() { dgx_state_free(u_); }
    double* data() const noexcept { return u_; }
    void upload(const std::vector<double>& h) { check(dgx_state_copy(c_, u_, h.data(), 1)); }
    void download(std::vector<double>& h) const { check(dgx_state_copy(c_, h.data(), u_, 0)); }

private:
    dgx_ctx* c_;
    double* u_ = nullptr;
};

// CompressibleDGSolverBase: the explicit SSP-RK3 path of dgfem's compressible solvers.
class CompressibleDGSolverBase : public DGAssembler {
public:
    using StateVector = std::vector<MatrixXd>;
    using InitialCondition = std::function<Vector4d(const Vector2d&)>;

    // CompressibleDGSolverBase::run_time_integration (src/solver/compressible_solver_base.cpp:201-338):
    // the initial condition projected, then SSP-RK3 steps while t < T_final; a frame is kept every
    // save_every steps and after the last step, each flattened to (n_elements, n_basis * 4); a step
    // that produces a NaN ends the loop.  The state stays on the GPU between steps: only the frames
    // are copied to the host.  dgfem's monitors (CFL, density range) every 10 steps are kept in
    // max_cfl_encountered() / last_density_range().
    std::vector<MatrixXd> solve(InitialCondition initial_condition, double T_final, double dt, int save_every = 1) {
        if (save_every < 1) throw std::invalid_argument("save_every must be positive");
        std::vector<double> h = project_flat(initial_condition);
        DeviceState u(*this);
        u.upload(h);
        std::vector<MatrixXd> frames;
        frames.push_back(flat_frame(h));
        double t = 0.0;
        int step = 0;
        max_cfl_ = 0.0;
        check(dgx_max_cfl(c_, u.data(), dt, &max_cfl_, nullptr));
        while (t < T_final) {
            if (step % save_every == 0 && step > 0) {
                u.download(h);
                frames.push_back(flat_frame(h));
            }
            if (step % 10 == 0) {
                double cfl = 0.0;
                check(dgx_max_cfl(c_, u.data(), dt, &cfl, nullptr));
                check(dgx_density_range(c_, u.data(), &rho_range_.first, &rho_range_.second, nullptr));
                if (cfl > max_cfl_) max_cfl_ = cfl;
            }
            check(dgx_rk3_step(c_, u.data(), dt, 1, nullptr));
            t += dt;
            ++step;
            int nonfinite = 0;
            const int rc = dgx_step_status(c_, &nonfinite, nullptr);
            if (rc != DGX_OK && rc != DGX_ERR_NONFINITE) check(rc);
            if (nonfinite) break;  // dgfem: "Solution contains NaN values; aborting integration"
        }
        if (step % save_every != 0) {
            u.download(h);
            frames.push_back(flat_frame(h));
        }
        steps_ = step;
        return frames;
    }

    // CompressibleDGSolverBase::project_initial_condition (:63-104): the functor at every volume
    // quadrature point, L2-projected on the GPU.
    StateVector project_initial_condition(const InitialCondition& u0) {
        StateVector out;
        unflatten(project_flat(u0), out);
        return out;
    }
    // apply_mass_inv, time_step_ssp_rk3, compute_max_cfl and compute_density_range on host states
    // (each call copies the state in and out; solve() keeps it on the device instead)
    StateVector apply_mass_inv(const StateVector& vec) {
        std::vector<double> a = flatten(vec), b(a.size());
        check(dgx_apply_mass_inv_host(c_, a.data(), b.data()));
        StateVector out;
        unflatten(b, out);
        return out;
    }
    StateVector time_step_ssp_rk3(const StateVector& u_n, double dt) {
        std::vector<double> u = flatten(u_n);
        check(dgx_rk3_step_host(c_, u.data(), dt, 1));
        StateVector out;
        unflatten(u, out);
        return out;
    }
    double compute_max_cfl(const StateVector& u, double dt) {
        std::vector<double> f = flatten(u);
        double cfl = 0.0;
        check(dgx_monitor_host(c_, f.data(), dt, &cfl, nullptr, nullptr, nullptr));
        return cfl;
    }
    std::pair<double, double> compute_density_range(const StateVector& u) {
        std::vector<double> f = flatten(u);
        double lo = 0.0, hi = 0.0;
        check(dgx_monitor_host(c_, f.data(), 0.0, nullptr, &lo, &hi, nullptr));
        return {lo, hi};
    }
    int steps_taken() const noexcept { return steps_; }
    double max_cfl_encountered() const noexcept { return max_cfl_; }
    std::pair<double, double> last_density_range() const noexcept { return rho_range_; }

protected:
    template <typename WeakFormT>
    CompressibleDGSolverBase(std::shared_ptr<DGMesh> mesh, std::shared_ptr<WeakFormT> wf, int precision)
        : DGAssembler(std::move(mesh), std::move(wf), precision) {}

    std::vector<double> project_flat(const InitialCondition& u0) {
        std::vector<double> xq((size_t)ne_ * nq_ * 2), uq((size_t)ne_ * nq_ * 4), u((size_t)ne_ * np_ * 4);
        check(dgx_quad_points(c_, xq.data()));
        for (size_t k = 0; k < (size_t)ne_ * nq_; ++k) {
            const Vector4d w = u0(Vector2d(xq[2 * k], xq[2 * k + 1]));
            for (int v = 0; v < 4; ++v) uq[4 * k + v] = w(v);
        }
        check(dgx_project_host(c_, uq.data(), u.data()));
        return u;
    }
    MatrixXd flat_frame(const std::vector<double>& h) const {  // flatten_frames (:340-368)
        MatrixXd m(ne_, np_ * 4);
        for (int e = 0; e < ne_; ++e)
            for (int k = 0; k < np_ * 4; ++k) m(e, k) = h[(size_t)e * np_ * 4 + k];
        return m;
    }

    double max_cfl_ = 0.0;
    std::pair<double, double> rho_range_{0.0, 0.0};
    int steps_ = 0;
};

// EulerDGSolver(mesh, gamma) / EulerDGSolver(mesh, weak_form) (dg_solver.hpp:262-276)
class EulerDGSolver : public CompressibleDGSolverBase {
public:
    explicit EulerDGSolver(std::shared_ptr<DGMesh> mesh, double gamma = 1.4, int precision = DGX_FP64)
        : CompressibleDGSolverBase(std::move(mesh), std::make_shared<EulerWeakFormulation>(gamma), precision) {}
    EulerDGSolver(std::shared_ptr<DGMesh> mesh, std::shared_ptr<EulerWeakFormulation> weak_form,
                  int precision = DGX_FP64)
        : CompressibleDGSolverBase(std::move(mesh), std::move(weak_form), precision) {}
};

// NavierStokesDGSolver(mesh, gamma, mu, Pr, sigma0) (dg_solver.hpp:281-296)
class NavierStokesDGSolver : public CompressibleDGSolverBase {
public:
    explicit NavierStokesDGSolver(std::shared_ptr<DGMesh> mesh, double gamma = 1.4, double dynamic_viscosity = 1.0e-3,
                                  double prandtl = 0.72, double penalty_prefactor = 5.0, int precision = DGX_FP64)
        : CompressibleDGSolverBase(std::move(mesh),
                                   std::make_shared<NavierStokesWeakFormulation>(gamma, dynamic_viscosity, prandtl,
                                                                                 penalty_prefactor),
                                   precision) {}
};

}  // namespace dgx_dgfem
