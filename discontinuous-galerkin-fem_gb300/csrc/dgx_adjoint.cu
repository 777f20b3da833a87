// Tangent-linear and adjoint entry points of include/dgx.h (FP64 contexts).
//
// Adjoint of one SSP-RK3 step (time_stepping.hpp:39-55), with J(u) = M^-1 dR/du and
// M symmetric, so J(u)^T x = (dR/du)^T (M^-1 x):
//   ubar2 = 2/3 ubar3 + 2/3 dt J(u2)^T ubar3
//   ubar1 = 1/4 ubar2 + 1/4 dt J(u1)^T ubar2
//   ubar_n = 1/3 ubar3 + 3/4 ubar2 + ubar1 + dt J(u_n)^T ubar1
// The gradient driver keeps a checkpoint every `checkpoint_every` steps; for each segment
// (last to first) it recomputes the segment forward, storing u^n, u1 and u2 of every step,
// then runs the adjoint steps backward through the stored states.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dg_adjoint.cuh"
#include "dgx_context.h"

using namespace dgx;

namespace {

template <int P, bool VISC>
int launch_jvp_t(const AdjArgs& a, const OpsHost& oh, cudaStream_t st) {
    JArgs<P, VISC> ka;
    ka.s = a;
    fill_ops<P, double>(oh, ka.o);
    for (int i = 0; i < n_basis(P); ++i)
        for (int j = 0; j < n_basis(P); ++j) ka.minv64[i][j] = oh.minv[i][j];
    if (cudaFuncSetAttribute(jvp_kernel<P, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)jvp_smem_bytes<P, VISC>()) != cudaSuccess)
        return -1;
    const int grid = (a.ne + TILE - 1) / TILE;
    jvp_kernel<P, VISC><<<grid, TILE, jvp_smem_bytes<P, VISC>(), st>>>(ka);
    return launch_status();
}

template <int P>
int launch_vjp_t(const AdjArgs& a, const OpsHost& oh, cudaStream_t st) {
    VArgs<P> ka;
    ka.s = a;
    fill_ops<P, double>(oh, ka.o);
    const int grid = (a.ne + TILE - 1) / TILE;
    vjp_kernel<P><<<grid, TILE, vjp_smem_bytes<P>(), st>>>(ka);
    return launch_status();
}

template <int P>
int configure_vjp_t() {
    return cudaFuncSetAttribute(vjp_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)vjp_smem_bytes<P>()) == cudaSuccess ? 0 : -1;
}

// J: device buffer of (n_blocks + 1) doubles (partial sums, then the total in the last slot)
template <int P>
int launch_kinetic_t(const AdjArgs& a, const OpsHost& oh, double* J, double* grad, cudaStream_t st) {
    VArgs<P> ka;
    ka.s = a;
    fill_ops<P, double>(oh, ka.o);
    const int grid = (a.ne + 127) / 128;
    kinetic_kernel<P><<<grid, 128, 0, st>>>(ka, J, grad);
    if (J) kinetic_sum_kernel<<<1, 32, 0, st>>>(J, grid, J + grid);
    return launch_status();
}

int launch_jvp(int p, bool visc, const AdjArgs& a, const OpsHost& o, cudaStream_t s) {
    switch (p * 2 + (visc ? 1 : 0)) {
    case 2: return launch_jvp_t<1, false>(a, o, s);
    case 3: return launch_jvp_t<1, true>(a, o, s);
    case 4: return launch_jvp_t<2, false>(a, o, s);
    case 5: return launch_jvp_t<2, true>(a, o, s);
    case 6: return launch_jvp_t<3, false>(a, o, s);
    case 7: return launch_jvp_t<3, true>(a, o, s);
    case 8: return launch_jvp_t<4, false>(a, o, s);
    case 9: return launch_jvp_t<4, true>(a, o, s);
    default: return -1;
    }
}

int launch_vjp(int p, const AdjArgs& a, const OpsHost& o, cudaStream_t s) {
    switch (p) {
    case 1: return configure_vjp_t<1>() || launch_vjp_t<1>(a, o, s);
    case 2: return configure_vjp_t<2>() || launch_vjp_t<2>(a, o, s);
    case 3: return configure_vjp_t<3>() || launch_vjp_t<3>(a, o, s);
    case 4: return configure_vjp_t<4>() || launch_vjp_t<4>(a, o, s);
    default: return -1;
    }
}

int launch_kinetic(int p, const AdjArgs& a, const OpsHost& o, double* J, double* grad, cudaStream_t s) {
    switch (p) {
    case 1: return launch_kinetic_t<1>(a, o, J, grad, s);
    case 2: return launch_kinetic_t<2>(a, o, J, grad, s);
    case 3: return launch_kinetic_t<3>(a, o, J, grad, s);
    case 4: return launch_kinetic_t<4>(a, o, J, grad, s);
    default: return -1;
    }
}

AdjArgs base(const dgx_ctx* c) {
    AdjArgs a{};
    a.ne = c->ne;
    a.geom = c->d_geom;
    a.conn = c->d_conn;
    a.bc = c->d_bc;
    a.gamma = c->prm.gamma;
    a.mu_visc = c->prm.mu;
    a.prandtl = c->prm.prandtl;
    a.sigma0 = c->prm.sigma0;
    a.minv_diag = c->minv_diag;
    return a;
}

int need_fp64(const dgx_ctx* c, const char* what) {
    if (c->prm.precision != DGX_FP64)
        return dgx::set_error(DGX_ERR_INVALID, std::string(what) + ": needs an FP64 context");
    return DGX_OK;
}

int need_adjoint(const dgx_ctx* c, const char* what) {
    if (int rc = need_fp64(c, what)) return rc;
    if (c->prm.physics != DGX_EULER)
        return dgx::set_error(DGX_ERR_INVALID, std::string(what) + ": the adjoint covers the Euler equations only");
    if (c->has_slip_wall)
        return dgx::set_error(DGX_ERR_INVALID, std::string(what) + ": slip-wall faces have no adjoint");
    return DGX_OK;
}

// the adjoint scratch: three states (ubar2, ubar1, mu)
int ensure_adjoint_buffers(dgx_ctx* c) {
    if (c->d_adj[0]) return DGX_OK;
    for (int k = 0; k < 3; ++k)
        if (cudaMalloc((void**)&c->d_adj[k], (c->nstate ? c->nstate : 1) * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return dgx::set_error(DGX_ERR_CUDA, "cudaMalloc failed for adjoint buffers");
        }
    return DGX_OK;
}

// one forward FP64 stage: out = a un + b (u + dt M^-1 R(u)) (a == 0: out = u + dt M^-1 R(u))
int fwd_stage(dgx_ctx* c, const double* u, const double* un, double* out, double a, double b, double dt,
              cudaStream_t s) {
    StepArgs st{};
    st.ne = c->ne;
    st.geom = c->d_geom;
    st.conn = c->d_conn;
    st.bc = c->d_bc;
    st.gamma = c->prm.gamma;
    st.mu = c->prm.mu;
    st.prandtl = c->prm.prandtl;
    st.sigma0 = c->prm.sigma0;
    st.order = c->prm.order;
    st.minv_diag = c->minv_diag;
    st.mode = MODE_STAGE;
    st.u = u;
    st.un = un;
    st.out = out;
    st.a = a;
    st.b = b;
    st.dt = dt;
    return launch_element_fp64(c->prm.order, c->prm.physics == DGX_NAVIER_STOKES, st, c->ops, s)
               ? dgx::set_error(DGX_ERR_CUDA, "forward stage launch failed")
               : DGX_OK;
}

// out = c0 x0 + c1 x1 + c2 x2 + cv (dR/du)^T M^-1 y, with M^-1 y written to mu_buf
int vjp_combo(dgx_ctx* c, const double* u, const double* y, double* mu_buf, double* out, const double* x0,
              double c0, const double* x1, double c1, const double* x2, double c2, double cv, cudaStream_t s) {
    if (launch_mass_inv(c->ne, c->prm.order, c->ops, c->d_geom, y, mu_buf, s))
        return dgx::set_error(DGX_ERR_CUDA, "mass inverse launch failed");
    AdjArgs a = base(c);
    a.u = u;
    a.mu = mu_buf;
    a.out = out;
    a.x0 = x0; a.c0 = c0;
    a.x1 = x1; a.c1 = c1;
    a.x2 = x2; a.c2 = c2;
    a.cv = cv;
    return launch_vjp(c->prm.order, a, c->ops, s) ? dgx::set_error(DGX_ERR_CUDA, "vjp launch failed") : DGX_OK;
}

// adjoint of one step given the stored stage states u_n, u1, u2; ubar in place
int adjoint_step(dgx_ctx* c, const double* un, const double* u1, const double* u2, double* ubar, double dt,
                 cudaStream_t s) {
    double* ub2 = c->d_adj[0];
    double* ub1 = c->d_adj[1];
    double* mu = c->d_adj[2];
    int rc = vjp_combo(c, u2, ubar, mu, ub2, ubar, 2.0 / 3.0, nullptr, 0, nullptr, 0, 2.0 / 3.0 * dt, s);
    if (!rc) rc = vjp_combo(c, u1, ub2, mu, ub1, ub2, 0.25, nullptr, 0, nullptr, 0, 0.25 * dt, s);
    if (!rc) rc = vjp_combo(c, un, ub1, mu, ubar, ubar, 1.0 / 3.0, ub2, 0.75, ub1, 1.0, dt, s);
    return rc;
}

}  // namespace

extern "C" int dgx_residual_jvp(dgx_ctx* c, const double* u, const double* du, double* dr, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_residual_jvp: triangle meshes only");
    if (!c || (c->ne && (!u || !du || !dr))) return dgx::set_error(DGX_ERR_INVALID, "dgx_residual_jvp: null argument");
    if (int rc = need_fp64(c, "dgx_residual_jvp")) return rc;
    if (c->ne == 0) return DGX_OK;
    AdjArgs a = base(c);
    a.mode = MODE_RESIDUAL;
    a.u = u;
    a.du = du;
    a.out = nullptr;
    a.dout = dr;
    if (launch_jvp(c->prm.order, c->prm.physics == DGX_NAVIER_STOKES, a, c->ops, (cudaStream_t)stream))
        return dgx::set_error(DGX_ERR_CUDA, "jvp launch failed");
    return DGX_OK;
}

extern "C" int dgx_residual_vjp(dgx_ctx* c, const double* u, const double* rbar, double* ubar, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_residual_vjp: triangle meshes only");
    if (!c || (c->ne && (!u || !rbar || !ubar))) return dgx::set_error(DGX_ERR_INVALID, "dgx_residual_vjp: null argument");
    if (int rc = need_adjoint(c, "dgx_residual_vjp")) return rc;
    if (c->ne == 0) return DGX_OK;
    AdjArgs a = base(c);
    a.u = u;
    a.mu = rbar;
    a.out = ubar;
    a.cv = 1.0;
    if (launch_vjp(c->prm.order, a, c->ops, (cudaStream_t)stream))
        return dgx::set_error(DGX_ERR_CUDA, "vjp launch failed");
    return DGX_OK;
}

extern "C" int dgx_rk3_step_tlm(dgx_ctx* c, double* u, double* du, double dt, int n_steps, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_rk3_step_tlm: triangle meshes only");
    if (!c || (c->ne && (!u || !du)) || n_steps < 0) return dgx::set_error(DGX_ERR_INVALID, "dgx_rk3_step_tlm: bad argument");
    if (int rc = need_fp64(c, "dgx_rk3_step_tlm")) return rc;
    if (c->ne == 0 || n_steps == 0) return DGX_OK;
    if (int rc = ensure_adjoint_buffers(c)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const bool visc = c->prm.physics == DGX_NAVIER_STOKES;
    double* u1 = c->d_u1;
    double* u2 = c->d_u2;
    double* d1 = c->d_adj[0];
    double* d2 = c->d_adj[1];
    AdjArgs a = base(c);
    a.mode = MODE_STAGE;
    a.dt = dt;
    for (int n = 0; n < n_steps; ++n) {
        a.u = u; a.du = du; a.out = u1; a.dout = d1; a.un = nullptr; a.dun = nullptr; a.a = 0.0; a.b = 1.0;
        if (launch_jvp(c->prm.order, visc, a, c->ops, s)) return dgx::set_error(DGX_ERR_CUDA, "jvp launch failed");
        a.u = u1; a.du = d1; a.out = u2; a.dout = d2; a.un = u; a.dun = du; a.a = 0.75; a.b = 0.25;
        if (launch_jvp(c->prm.order, visc, a, c->ops, s)) return dgx::set_error(DGX_ERR_CUDA, "jvp launch failed");
        a.u = u2; a.du = d2; a.out = u; a.dout = du; a.un = u; a.dun = du; a.a = 1.0 / 3.0; a.b = 2.0 / 3.0;
        if (launch_jvp(c->prm.order, visc, a, c->ops, s)) return dgx::set_error(DGX_ERR_CUDA, "jvp launch failed");
    }
    return DGX_OK;
}

extern "C" int dgx_rk3_step_adjoint(dgx_ctx* c, const double* u_n, double* ubar, double dt, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_rk3_step_adjoint: triangle meshes only");
    if (!c || (c->ne && (!u_n || !ubar))) return dgx::set_error(DGX_ERR_INVALID, "dgx_rk3_step_adjoint: null argument");
    if (int rc = need_adjoint(c, "dgx_rk3_step_adjoint")) return rc;
    if (c->ne == 0) return DGX_OK;
    if (int rc = ensure_adjoint_buffers(c)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = fwd_stage(c, u_n, nullptr, c->d_u1, 0.0, 1.0, dt, s);
    if (!rc) rc = fwd_stage(c, c->d_u1, u_n, c->d_u2, 0.75, 0.25, dt, s);
    if (!rc) rc = adjoint_step(c, u_n, c->d_u1, c->d_u2, ubar, dt, s);
    return rc;
}

extern "C" int dgx_kinetic_energy(dgx_ctx* c, const double* u, double* J, double* grad, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_kinetic_energy: triangle meshes only");
    if (!c || (c->ne && !u)) return dgx::set_error(DGX_ERR_INVALID, "dgx_kinetic_energy: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (c->ne == 0) {
        if (J) *J = 0.0;
        return DGX_OK;
    }
    const int nblk = (c->ne + 127) / 128;
    if (J && !c->d_kin) {
        if (cudaMalloc((void**)&c->d_kin, sizeof(double) * (nblk + 1)) != cudaSuccess) {
            cudaGetLastError();
            return dgx::set_error(DGX_ERR_CUDA, "cudaMalloc failed for the objective reduction");
        }
    }
    AdjArgs a = base(c);
    a.u = u;
    if (launch_kinetic(c->prm.order, a, c->ops, J ? c->d_kin : nullptr, grad, s))
        return dgx::set_error(DGX_ERR_CUDA, "kinetic energy launch failed");
    if (J) {
        if (cudaMemcpyAsync(J, c->d_kin + nblk, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return dgx::set_error(DGX_ERR_CUDA, "kinetic energy read-back failed");
    }
    return DGX_OK;
}

extern "C" int dgx_kinetic_energy_gradient(dgx_ctx* c, const double* u0, double dt, int n_steps,
                                           int checkpoint_every, double* J, double* grad, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_kinetic_energy_gradient: triangle meshes only");
    if (!c || (c->ne && (!u0 || !grad)) || n_steps < 0 || checkpoint_every < 1)
        return dgx::set_error(DGX_ERR_INVALID, "dgx_kinetic_energy_gradient: bad argument");
    if (int rc = need_adjoint(c, "dgx_kinetic_energy_gradient")) return rc;
    if (c->ne == 0) return DGX_OK;
    if (int rc = ensure_adjoint_buffers(c)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t sb = c->nstate * sizeof(double);
    const int nseg = (n_steps + checkpoint_every - 1) / checkpoint_every;
    const int seg_len = n_steps < checkpoint_every ? n_steps : checkpoint_every;
    // storage: nseg + 1 checkpoints, and 3 states per step of one segment
    std::vector<double*> ck(nseg + 1, nullptr);
    std::vector<double*> st(3 * (size_t)seg_len + 1, nullptr);
    auto release = [&]() {
        for (double* p : ck) cudaFree(p);
        for (double* p : st) cudaFree(p);
    };
    for (auto& p : ck)
        if (cudaMalloc((void**)&p, sb) != cudaSuccess) {
            cudaGetLastError();
            release();
            return dgx::set_error(DGX_ERR_CUDA, "cudaMalloc failed for checkpoints");
        }
    for (auto& p : st)
        if (cudaMalloc((void**)&p, sb) != cudaSuccess) {
            cudaGetLastError();
            release();
            return dgx::set_error(DGX_ERR_CUDA, "cudaMalloc failed for segment states");
        }
    int rc = DGX_OK;
    // forward sweep keeping checkpoints
    if (cudaMemcpyAsync(ck[0], u0, sb, cudaMemcpyDeviceToDevice, s) != cudaSuccess) rc = DGX_ERR_CUDA;
    for (int g = 0; g < nseg && !rc; ++g) {
        const int n0 = g * checkpoint_every, n1 = std::min(n_steps, n0 + checkpoint_every);
        if (cudaMemcpyAsync(ck[g + 1], ck[g], sb, cudaMemcpyDeviceToDevice, s) != cudaSuccess) rc = DGX_ERR_CUDA;
        for (int n = n0; n < n1 && !rc; ++n) {
            rc = fwd_stage(c, ck[g + 1], nullptr, c->d_u1, 0.0, 1.0, dt, s);
            if (!rc) rc = fwd_stage(c, c->d_u1, ck[g + 1], c->d_u2, 0.75, 0.25, dt, s);
            if (!rc) rc = fwd_stage(c, c->d_u2, ck[g + 1], ck[g + 1], 1.0 / 3.0, 2.0 / 3.0, dt, s);
        }
    }
    // objective and its gradient at u(T) -> ubar
    if (!rc) rc = dgx_kinetic_energy(c, ck[nseg], J, grad, stream);
    // backward sweep: recompute each segment storing (u_n, u1, u2), then adjoint steps
    for (int g = nseg - 1; g >= 0 && !rc; --g) {
        const int n0 = g * checkpoint_every, n1 = std::min(n_steps, n0 + checkpoint_every), m = n1 - n0;
        if (cudaMemcpyAsync(st[0], ck[g], sb, cudaMemcpyDeviceToDevice, s) != cudaSuccess) rc = DGX_ERR_CUDA;
        for (int k = 0; k < m && !rc; ++k) {
            double* un = st[3 * k];
            double* u1 = st[3 * k + 1];
            double* u2 = st[3 * k + 2];
            double* nx = st[3 * k + 3];
            rc = fwd_stage(c, un, nullptr, u1, 0.0, 1.0, dt, s);
            if (!rc) rc = fwd_stage(c, u1, un, u2, 0.75, 0.25, dt, s);
            if (!rc) rc = fwd_stage(c, u2, un, nx, 1.0 / 3.0, 2.0 / 3.0, dt, s);
        }
        for (int k = m - 1; k >= 0 && !rc; --k) rc = adjoint_step(c, st[3 * k], st[3 * k + 1], st[3 * k + 2], grad, dt, s);
    }
    if (!rc && cudaStreamSynchronize(s) != cudaSuccess) rc = dgx::set_error(DGX_ERR_CUDA, "gradient sweep failed");
    release();
    if (rc == DGX_ERR_CUDA && std::string(dgx_last_error()).empty()) dgx::set_error(rc, "gradient sweep failed");
    return rc;
}

// ---------------------------------------------------------------- binomial checkpointing
// The reverse sweep of n SSP-RK3 steps with s snapshot states beside the stored start state:
// F(n, s) = the fewest forward steps it recomputes, F(1, s) = 0 (one adjoint step recomputes
// its own two stages), F(n, 0) = n (n - 1) / 2 (every step re-advanced from the start), and
// F(n, s) = min over k of k + F(n - k, s - 1) + F(k, s): advance k steps into a snapshot, reverse
// the n - k steps after it with one snapshot fewer, then the k steps before it.  Solved exactly
// by dynamic programming; its minima are the binomial schedules of Griewank's revolve.
namespace {
struct BinomialSchedule {
    int N = 0, S = 0;
    std::vector<long long> F;
    std::vector<int> K;
    size_t at(int n, int s) const { return (size_t)n * (S + 1) + s; }
    void build(int n_steps, int snaps) {
        N = n_steps;
        S = snaps;
        F.assign((size_t)(N + 1) * (S + 1), 0);
        K.assign(F.size(), 1);
        for (int n = 1; n <= N; ++n) F[at(n, 0)] = (long long)n * (n - 1) / 2;
        for (int sn = 1; sn <= S; ++sn)
            for (int n = 2; n <= N; ++n) {
                long long best = -1;
                int bk = 1;
                for (int k = 1; k < n; ++k) {
                    const long long v = k + F[at(n - k, sn - 1)] + F[at(k, sn)];
                    if (best < 0 || v < best) {
                        best = v;
                        bk = k;
                    }
                }
                F[at(n, sn)] = best;
                K[at(n, sn)] = bk;
            }
    }
};

struct BinomialRun {
    dgx_ctx* c;
    double dt;
    cudaStream_t st;
    const BinomialSchedule* plan;
    std::vector<double*> snap;  // snap[l - 1]: the snapshot of recursion level l
    double* work;               // the re-advanced state of the levels without snapshots
    double* grad;
    long long recomputed = 0;

    int step(double* x) {  // one SSP-RK3 step in place
        int rc = fwd_stage(c, x, nullptr, c->d_u1, 0.0, 1.0, dt, st);
        if (!rc) rc = fwd_stage(c, c->d_u1, x, c->d_u2, 0.75, 0.25, dt, st);
        if (!rc) rc = fwd_stage(c, c->d_u2, x, x, 1.0 / 3.0, 2.0 / 3.0, dt, st);
        return rc;
    }
    int adjoint_at(const double* x) {  // the cotangent across the step that starts at x
        int rc = fwd_stage(c, x, nullptr, c->d_u1, 0.0, 1.0, dt, st);
        if (!rc) rc = fwd_stage(c, c->d_u1, x, c->d_u2, 0.75, 0.25, dt, st);
        if (!rc) rc = adjoint_step(c, x, c->d_u1, c->d_u2, grad, dt, st);
        return rc;
    }
    int copy(double* dst, const double* src) {
        return cudaMemcpyAsync(dst, src, c->nstate * sizeof(double), cudaMemcpyDeviceToDevice, st) == cudaSuccess
                   ? DGX_OK
                   : dgx::set_error(DGX_ERR_CUDA, "state copy failed");
    }
    // reverses the n steps after state ua (left unchanged) with sn snapshots
    int reverse(const double* ua, int n, int sn) {
        if (n == 1) return adjoint_at(ua);
        if (sn == 0) {
            for (int j = n - 1; j >= 0; --j) {
                if (int rc = copy(work, ua)) return rc;
                for (int t = 0; t < j; ++t)
                    if (int rc = step(work)) return rc;
                recomputed += j;
                if (int rc = adjoint_at(work)) return rc;
            }
            return DGX_OK;
        }
        const int k = plan->K[plan->at(n, sn)];
        double* sp = snap[sn - 1];
        if (int rc = copy(sp, ua)) return rc;
        for (int t = 0; t < k; ++t)
            if (int rc = step(sp)) return rc;
        recomputed += k;
        if (int rc = reverse(sp, n - k, sn - 1)) return rc;
        return reverse(ua, k, sn);
    }
};
}  // namespace

extern "C" int dgx_kinetic_energy_gradient_binomial(dgx_ctx* c, const double* u0, double dt, int n_steps,
                                                    int n_snapshots, double* J, double* grad, long long* stats,
                                                    void* stream) {
    if (c && c->nvpe == 4)
        return dgx::set_error(DGX_ERR_INVALID, "dgx_kinetic_energy_gradient_binomial: triangle meshes only");
    if (!c || (c->ne && (!u0 || !grad)) || n_steps < 0 || n_snapshots < 0)
        return dgx::set_error(DGX_ERR_INVALID, "dgx_kinetic_energy_gradient_binomial: bad argument");
    // the schedule costs O(n_steps^2 n_snapshots) host operations
    if ((double)n_steps * n_steps * (n_snapshots + 1) > 4.0e9)
        return dgx::set_error(DGX_ERR_INVALID,
                              "dgx_kinetic_energy_gradient_binomial: n_steps^2 * (n_snapshots + 1) above 4e9; "
                              "use dgx_kinetic_energy_gradient's uniform checkpoints");
    if (int rc = need_adjoint(c, "dgx_kinetic_energy_gradient_binomial")) return rc;
    if (c->ne == 0) return DGX_OK;
    if (int rc = ensure_adjoint_buffers(c)) return rc;
    const int snaps = std::min(n_snapshots, std::max(n_steps - 1, 0));
    BinomialSchedule plan;
    plan.build(n_steps, snaps);
    BinomialRun run{c, dt, (cudaStream_t)stream, &plan, std::vector<double*>(snaps, nullptr), nullptr, grad};
    const size_t sb = c->nstate * sizeof(double);
    auto release = [&]() {
        for (double* p : run.snap) cudaFree(p);
        cudaFree(run.work);
    };
    if (cudaMalloc((void**)&run.work, sb) != cudaSuccess) {
        cudaGetLastError();
        return dgx::set_error(DGX_ERR_CUDA, "cudaMalloc failed for the work state");
    }
    for (auto& p : run.snap)
        if (cudaMalloc((void**)&p, sb) != cudaSuccess) {
            cudaGetLastError();
            release();
            return dgx::set_error(DGX_ERR_CUDA, "cudaMalloc failed for snapshots");
        }
    // forward sweep to u(T) for the objective and its gradient, then the reverse sweep
    int rc = run.copy(run.work, u0);
    for (int n = 0; n < n_steps && !rc; ++n) rc = run.step(run.work);
    if (!rc) rc = dgx_kinetic_energy(c, run.work, J, grad, stream);
    if (!rc && n_steps > 0) rc = run.reverse(u0, n_steps, snaps);
    if (!rc && cudaStreamSynchronize(run.st) != cudaSuccess) rc = dgx::set_error(DGX_ERR_CUDA, "gradient sweep failed");
    release();
    if (stats) {
        stats[0] = run.recomputed;                                   // forward steps of the reverse sweep
        stats[1] = snaps + 1;                                        // states held besides u0 and the stages
        stats[2] = n_steps > 0 ? plan.F[plan.at(n_steps, snaps)] : 0;  // the schedule's optimum
    }
    return rc;
}
