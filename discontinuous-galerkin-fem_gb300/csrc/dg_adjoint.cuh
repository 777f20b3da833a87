// Differentiation of the FP64 DG residual and SSP-RK3 step.
//
//  * Tangent-linear (JVP): the forward element body run on dual numbers (value,
//    derivative), so it is exactly the derivative of the code that computes the residual.
//  * Adjoint (VJP): hand-written reverse of the Euler volume term and the Rusanov faces.
//    It uses a pull formulation, each element gathering its cotangent from its own faces and its
//    neighbours' faces.  Because the Rusanov flux is antisymmetric,
//    H(U_n, U_e, -n) = -H(U_e, U_n, n), the neighbour's face term that depends on this
//    element is -dH/dU_L(U_e, U_n, n)^T lambda_nbr, so both face terms combine into one
//    transposed Jacobian-vector product per face point:
//        ubar_e += phi_f^T dH/dU_L(U_e, U_n, n)^T (lambdaH_e - lambdaH_n),
//        lambdaH_x = -w (h/2) phi^T mu_x,   mu = M^-1 * cotangent.
//    Ties of the Rusanov wave-speed maximum (a set of measure zero) take the branch the
//    forward code takes.  The viscous terms and slip-wall faces have no adjoint here.
#pragma once

#include "dg_element.cuh"

namespace dgx {

// ---------------------------------------------------------------- dual numbers
struct Dual {
    double v, d;
    __host__ __device__ Dual() : v(0.0), d(0.0) {}
    __host__ __device__ Dual(double x) : v(x), d(0.0) {}
    __host__ __device__ Dual(double x, double dx) : v(x), d(dx) {}
    __device__ Dual& operator+=(const Dual& o) { v += o.v; d += o.d; return *this; }
    __device__ Dual& operator-=(const Dual& o) { v -= o.v; d -= o.d; return *this; }
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return Dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return Dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double r = 1.0 / b.v;
    const double q = a.v * r;
    return Dual(q, (a.d - q * b.d) * r);
}
__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(Dual a, Dual b) { return a.v > b.v; }
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? -a : a; }
template <>
__device__ __forceinline__ Dual rcp_<Dual>(Dual x) {
    const double r = 1.0 / x.v;
    return Dual(r, -x.d * r * r);
}
template <>
__device__ __forceinline__ Dual sqrt_<Dual>(Dual x) {
    const double s = sqrt(x.v);
    return Dual(s, s > 0.0 ? 0.5 * x.d / s : 0.0);
}

// ---------------------------------------------------------------- arguments
struct AdjArgs {
    int ne, mode;              // Mode (jvp); vjp ignores it
    const double* u;           // state (stage state of the linearisation)
    const double* du;          // jvp: tangent of u
    double* out;               // jvp: value output; vjp: cotangent output
    double* dout;              // jvp: tangent output
    const double* un;          // jvp MODE_STAGE: u^n
    const double* dun;         // jvp MODE_STAGE: tangent of u^n
    double dt, a, b;           // jvp MODE_STAGE combination (as StepArgs)
    const double* mu;          // vjp: M^-1 applied to the incoming cotangent
    const double* x0;          // vjp epilogue: out = c0 x0 + c1 x1 + c2 x2 + cv * (dR/du)^T mu
    const double* x1;
    const double* x2;
    double c0, c1, c2, cv;
    const ElemGeom* geom;
    const ElemConn* conn;
    const BCSlot* bc;
    double gamma, mu_visc, prandtl, sigma0;
    int minv_diag;
};

template <int P, bool VISC>
struct JArgs {
    AdjArgs s;
    Ops<P, double> o;
    double minv64[n_basis(P)][n_basis(P)];
};

template <int P>
struct VArgs {
    AdjArgs s;
    Ops<P, double> o;
};

// ---------------------------------------------------------------- JVP kernel
template <int P, bool VISC>
__global__ void __launch_bounds__(TILE) jvp_kernel(const __grid_constant__ JArgs<P, VISC> ka) {
    constexpr int NP = n_basis(P), NB = NP * NV, STR = NB + 1;
    const AdjArgs& s = ka.s;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Dual* sU = reinterpret_cast<Dual*>(smem_raw);
    const int e0 = blockIdx.x * TILE;
    const int nloc = min(TILE, s.ne - e0);
    const int tl = threadIdx.x;
    const bool active = tl < nloc;
    const int e = e0 + tl;
    for (int g = tl; g < nloc * NB; g += TILE) {
        const int el = g / NB;
        sU[el * STR + (g - el * NB)] = Dual(s.u[(size_t)e0 * NB + g], s.du[(size_t)e0 * NB + g]);
    }
    __syncthreads();
    Dual R[NP][NV];
    if (active) {
        const double* uu = s.u;
        const double* dd = s.du;
        auto getrow = [uu, dd](int nb, int i, Dual c[4]) {
            const double* p = uu + (size_t)nb * NB + i * NV;
            const double* q = dd + (size_t)nb * NB + i * NV;
            for (int v = 0; v < NV; ++v) c[v] = Dual(p[v], q[v]);
        };
        const double kappa = VISC ? s.mu_visc * s.gamma / (s.prandtl * (s.gamma - 1.0)) : 0.0;
        element_residual<P, Dual, VISC, false, false>(ka.o, (const LiftOps<P, double>*)nullptr, sU + tl * STR, sU,
                                                      e0, nloc, s.geom[e], s.conn[e], s.bc, s.geom, Dual(s.gamma),
                                                      Dual(s.mu_visc), Dual(kappa), Dual(s.sigma0), getrow, R);
    }
    __syncthreads();
    double* sV = reinterpret_cast<double*>(smem_raw);  // [TILE][STR] values
    double* sT = sV + TILE * STR;                       // [TILE][STR] tangents
    if (active) {
        if (s.mode == MODE_RESIDUAL) {
            for (int i = 0; i < NP; ++i)
                for (int v = 0; v < NV; ++v) {
                    sV[tl * STR + i * NV + v] = R[i][v].v;
                    sT[tl * STR + i * NV + v] = R[i][v].d;
                }
        } else {
            const double ij = 1.0 / s.geom[e].detJ;
            for (int i = 0; i < NP; ++i)
                for (int v = 0; v < NV; ++v) {
                    double av = 0.0, ad = 0.0;
                    for (int k = 0; k < NP; ++k) {
                        if (s.minv_diag && k != i) continue;
                        av += ka.minv64[i][k] * R[k][v].v;
                        ad += ka.minv64[i][k] * R[k][v].d;
                    }
                    sV[tl * STR + i * NV + v] = av * ij;
                    sT[tl * STR + i * NV + v] = ad * ij;
                }
        }
    }
    __syncthreads();
    const size_t base = (size_t)e0 * NB;
    for (int g = tl; g < nloc * NB; g += TILE) {
        const int el = g / NB;
        const double lv = sV[el * STR + (g - el * NB)], ld = sT[el * STR + (g - el * NB)];
        if (s.mode != MODE_STAGE) {
            if (s.out) s.out[base + g] = lv;
            s.dout[base + g] = ld;
        } else if (s.a == 0.0) {
            s.out[base + g] = s.u[base + g] + s.dt * lv;
            s.dout[base + g] = s.du[base + g] + s.dt * ld;
        } else {
            const double tv = s.u[base + g] + s.dt * lv, td = s.du[base + g] + s.dt * ld;
            const double r = s.a * s.un[base + g] + s.b * tv;
            const double rd = s.a * s.dun[base + g] + s.b * td;
            s.out[base + g] = r;
            s.dout[base + g] = rd;
        }
    }
}

// ---------------------------------------------------------------- VJP pieces
// Reverse of euler_flux: given Fbar, Gbar and extra adjoints on the primitives (u, v, p,
// 1/rho), accumulate the cotangent of the conserved state U.
__device__ __forceinline__ void euler_flux_vjp(const double U[4], double gm1, const double Fb[4],
                                               const double Gb[4], double ub, double vb, double pb,
                                               double rib, double Ub[4]) {
    const double rho = U[0], E = U[3];
    const double ri = 1.0 / rho;
    const double u = U[1] * ri, v = U[2] * ri;
    const double q = u * u + v * v;
    const double p = gm1 * (E - 0.5 * rho * q);
    double rhob = 0.0, Eb = 0.0, mxb = Fb[0], myb = Gb[0];
    // F1 = rho u u + p, G2 = rho v v + p
    rhob += Fb[1] * u * u + Gb[2] * v * v;
    ub += 2.0 * Fb[1] * rho * u;
    vb += 2.0 * Gb[2] * rho * v;
    pb += Fb[1] + Gb[2];
    // F2 = G1 = rho u v
    const double c = Fb[2] + Gb[1];
    rhob += c * u * v;
    ub += c * rho * v;
    vb += c * rho * u;
    // F3 = u (E + p), G3 = v (E + p)
    ub += Fb[3] * (E + p);
    vb += Gb[3] * (E + p);
    Eb += Fb[3] * u + Gb[3] * v;
    pb += Fb[3] * u + Gb[3] * v;
    // p = gm1 (E - 1/2 rho q)
    Eb += gm1 * pb;
    rhob -= 0.5 * gm1 * q * pb;
    const double qb = -0.5 * gm1 * rho * pb;
    ub += 2.0 * u * qb;
    vb += 2.0 * v * qb;
    // u = mx ri, v = my ri, ri = 1/rho
    mxb += ub * ri;
    myb += vb * ri;
    rib += ub * U[1] + vb * U[2];
    rhob -= rib * ri * ri;
    Ub[0] += rhob;
    Ub[1] += mxb;
    Ub[2] += myb;
    Ub[3] += Eb;
}

// Cotangent of U_L of the Rusanov flux H(U_L, U_R, n) (rusanov in dg_physics.cuh).
__device__ __forceinline__ void rusanov_vjp_L(const double UL[4], const double UR[4], double nx, double ny,
                                              double gamma, const double Hb[4], double ULb[4]) {
    const double gm1 = gamma - 1.0;
    double FL[4], GL[4], FR[4], GR[4], uL, vL, pL, riL, uR, vR, pR, riR;
    euler_flux<double>(UL, gm1, FL, GL, uL, vL, pL, riL);
    euler_flux<double>(UR, gm1, FR, GR, uR, vR, pR, riR);
    const double cL = sqrt(gamma * pL * riL), cR = sqrt(gamma * pR * riR);
    const double unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
    const double aL = ::fabs(unL) + cL, aR = ::fabs(unR) + cR;
    const double hs = 0.5 * (aL < aR ? aR : aL);
    double Fb[4], Gb[4], hsb = 0.0;
    for (int v = 0; v < 4; ++v) {
        Fb[v] = 0.5 * nx * Hb[v];
        Gb[v] = 0.5 * ny * Hb[v];
        ULb[v] += hs * Hb[v];
        hsb -= Hb[v] * (UR[v] - UL[v]);
    }
    double ub = 0.0, vb = 0.0, pb = 0.0, rib = 0.0;
    if (!(aL < aR)) {  // the L side sets the wave speed
        const double ab = 0.5 * hsb;
        const double unb = unL >= 0.0 ? ab : -ab;
        ub += unb * nx;
        vb += unb * ny;
        if (cL > 0.0) {
            const double tb = ab / (2.0 * cL);  // c = sqrt(gamma p ri)
            pb += tb * gamma * riL;
            rib += tb * gamma * pL;
        }
    }
    euler_flux_vjp(UL, gm1, Fb, Gb, ub, vb, pb, rib, ULb);
}

// ---------------------------------------------------------------- VJP kernel
// out = c0 x0 + c1 x1 + c2 x2 + cv (dR/du)^T mu, R the residual of assemble_euler_residual.
template <int P>
__global__ void __launch_bounds__(TILE) vjp_kernel(const __grid_constant__ VArgs<P> ka) {
    constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1, NB = NP * NV, STR = NB + 1;
    const AdjArgs& s = ka.s;
    const Ops<P, double>& o = ka.o;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sU = reinterpret_cast<double*>(smem_raw);  // [TILE][STR] state
    double* sM = sU + TILE * STR;                       // [TILE][STR] mu
    const int e0 = blockIdx.x * TILE;
    const int nloc = min(TILE, s.ne - e0);
    const int tl = threadIdx.x;
    const bool active = tl < nloc;
    const int e = e0 + tl;
    const size_t base = (size_t)e0 * NB;
    for (int g = tl; g < nloc * NB; g += TILE) {
        const int el = g / NB;
        sU[el * STR + (g - el * NB)] = __ldg(s.u + base + g);
        sM[el * STR + (g - el * NB)] = __ldg(s.mu + base + g);
    }
    __syncthreads();
    double Ub[NP][NV];
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) Ub[i][v] = 0.0;
    if (active) {
        const double gamma = s.gamma, gm1 = gamma - 1.0;
        const ElemGeom& G = s.geom[e];
        const double A00 = G.A[0], A01 = G.A[1], A10 = G.A[2], A11 = G.A[3], detJ = G.detJ;
        const double* Ue = sU + tl * STR;
        const double* Me = sM + tl * STR;
        // volume: R_i += sum_q dr[q][i] Fr_q + ds[q][i] Fs_q
#pragma unroll 1
        for (int q = 0; q < NQ; ++q) {
            double U[4] = {0, 0, 0, 0}, lr[4] = {0, 0, 0, 0}, ls[4] = {0, 0, 0, 0};
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    U[v] += o.phi[q][i] * Ue[i * NV + v];
                    lr[v] += o.dr[q][i] * Me[i * NV + v];
                    ls[v] += o.ds[q][i] * Me[i * NV + v];
                }
            const double w = o.wq[q] * detJ;
            double Fb[4], Gb[4], Uq[4] = {0, 0, 0, 0};
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                Fb[v] = w * (A00 * lr[v] + A01 * ls[v]);
                Gb[v] = w * (A10 * lr[v] + A11 * ls[v]);
            }
            euler_flux_vjp(U, gm1, Fb, Gb, 0.0, 0.0, 0.0, 0.0, Uq);
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) Ub[i][v] += o.phi[q][i] * Uq[v];
        }
        // faces
        const ElemConn C = s.conn[e];
#pragma unroll 1
        for (int f = 0; f < 3; ++f) {
            const int nb = C.nbr[f];
            if (nb == NBR_SKIP) continue;
            const int fl = (C.flags >> (4 * f)) & 15;
            const int nf = fl & 3;
            const bool rev = (fl >> 2) & 1;
            const double nx = G.n[f][0], ny = G.n[f][1], hF = G.h[f];
            const double* Un_p = nullptr;
            const double* Mn_p = nullptr;
            BCSlot bc;
            bc.type = -1;
            if (nb >= 0) {
                if (nb >= e0 && nb < e0 + nloc) {
                    Un_p = sU + (nb - e0) * STR;
                    Mn_p = sM + (nb - e0) * STR;
                } else {
                    Un_p = s.u + (size_t)nb * NB;
                    Mn_p = s.mu + (size_t)nb * NB;
                }
            } else {
                bc = s.bc[-1 - nb];
            }
#pragma unroll 1
            for (int j = 0; j < NFQ; ++j) {
                const int k = rev ? NFQ - 1 - j : j;
                const double sc = o.wf[j] * hF * 0.5;
                double Uo[4] = {0, 0, 0, 0}, Un[4] = {0, 0, 0, 0}, hb[4] = {0, 0, 0, 0};
#pragma unroll
                for (int i = 0; i < NP; ++i)
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        Uo[v] += o.phif[f][j][i] * Ue[i * NV + v];
                        hb[v] -= sc * o.phif[f][j][i] * Me[i * NV + v];
                    }
                if (nb >= 0) {
#pragma unroll
                    for (int i = 0; i < NP; ++i)
#pragma unroll
                        for (int v = 0; v < NV; ++v) {
                            Un[v] += o.phif[nf][k][i] * Un_p[i * NV + v];
                            hb[v] += sc * o.phif[nf][k][i] * Mn_p[i * NV + v];  // - lambdaH_n
                        }
                } else if (bc.type == DGX_BC_FAR_FIELD) {
#pragma unroll
                    for (int v = 0; v < 4; ++v) Un[v] = bc.value[v];
                } else if (bc.type == DGX_BC_NO_SLIP_WALL) {
                    p2c<double>(bc.value, gamma, Un);
                } else {
                    continue;
                }
                double Ob[4] = {0, 0, 0, 0};
                rusanov_vjp_L(Uo, Un, nx, ny, gamma, hb, Ob);
#pragma unroll
                for (int i = 0; i < NP; ++i)
#pragma unroll
                    for (int v = 0; v < NV; ++v) Ub[i][v] += o.phif[f][j][i] * Ob[v];
            }
        }
    }
    __syncthreads();
    if (active) {
#pragma unroll
        for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int v = 0; v < NV; ++v) sU[tl * STR + i * NV + v] = Ub[i][v];
    }
    __syncthreads();
    for (int g = tl; g < nloc * NB; g += TILE) {
        const int el = g / NB;
        double r = s.cv * sU[el * STR + (g - el * NB)];
        if (s.x0) r += s.c0 * s.x0[base + g];
        if (s.x1) r += s.c1 * s.x1[base + g];
        if (s.x2) r += s.c2 * s.x2[base + g];
        s.out[base + g] = r;
    }
}

// ---------------------------------------------------------------- kinetic energy
// J = sum_e sum_q w_q |J_e| ((rho u)^2 + (rho v)^2) / (2 rho) at the volume points, and
// its gradient with respect to the modal state.
template <int P>
__global__ void kinetic_kernel(const __grid_constant__ VArgs<P> ka, double* J, double* grad) {
    constexpr int NP = n_basis(P), NQ = n_quad(P), NB = NP * NV;
    const AdjArgs& s = ka.s;
    const Ops<P, double>& o = ka.o;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (e < s.ne) {
        const double* ue = s.u + (size_t)e * NB;
        const double dj = s.geom[e].detJ;
        double g[NP][NV];
        for (int i = 0; i < NP; ++i)
            for (int v = 0; v < NV; ++v) g[i][v] = 0.0;
        for (int q = 0; q < NQ; ++q) {
            double U[4] = {0, 0, 0, 0};
            for (int i = 0; i < NP; ++i)
                for (int v = 0; v < NV; ++v) U[v] += o.phi[q][i] * ue[i * NV + v];
            const double w = o.wq[q] * dj, ri = 1.0 / U[0];
            const double m2 = U[1] * U[1] + U[2] * U[2];
            acc += w * 0.5 * m2 * ri;
            const double dU[4] = {-0.5 * w * m2 * ri * ri, w * U[1] * ri, w * U[2] * ri, 0.0};
            for (int i = 0; i < NP; ++i)
                for (int v = 0; v < NV; ++v) g[i][v] += o.phi[q][i] * dU[v];
        }
        if (grad)
            for (int i = 0; i < NP; ++i)
                for (int v = 0; v < NV; ++v) grad[(size_t)e * NB + i * NV + v] = g[i][v];
    }
    if (J) {  // per-block partial sums, combined in a fixed order by kinetic_sum_kernel
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        __shared__ double warp_sums[32];
        if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double b = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += warp_sums[w];
            J[blockIdx.x] = b;
        }
    }
}

// Compensated (Kahan) sum of the per-block partial sums, in block order: the objective is
// a deterministic function of the state.
__global__ void kinetic_sum_kernel(const double* partial, int n, double* J) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0, c = 0.0;
    for (int i = 0; i < n; ++i) {
        const double y = partial[i] - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    *J = s;
}

template <int P, bool VISC>
inline size_t jvp_smem_bytes() {
    return (size_t)TILE * (n_basis(P) * NV + 1) * sizeof(Dual);
}
template <int P>
inline size_t vjp_smem_bytes() {
    return (size_t)2 * TILE * (n_basis(P) * NV + 1) * sizeof(double);
}

}  // namespace dgx
