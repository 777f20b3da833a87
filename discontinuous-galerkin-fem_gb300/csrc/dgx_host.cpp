// Host side of the C ABI (include/dgx.h): mesh connectivity with dgfem's semantics,
// reference-element operators, per-element geometry records, the device-resident
// context and the stream-ordered entry points.
#include "../../include/dgx.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <string>
#include <unordered_set>
#include <vector>

#include "dgx_context.h"
#include "dgx_internal.h"
#include "quad_tables.inc"

using namespace dgx;

// ------------------------------------------------------------------ errors
static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CUDA_OK(x)                                                                    \
    do {                                                                              \
        cudaError_t e_ = (x);                                                         \
        if (e_ != cudaSuccess)                                                        \
            return fail(DGX_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

extern "C" const char* dgx_last_error(void) { return g_err.c_str(); }

int dgx::set_error(int code, const std::string& msg) { return fail(code, msg); }
extern "C" const char* dgx_version(void) { return "dgx 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ bases
// MonomialBasisTriangle (src/basis/monomial.cpp:30-72): x^i y^j ordered by total degree,
// then i ascending.
static double ipow(double x, int n) { return n == 0 ? 1.0 : std::pow(x, (double)n); }

static void monomial(int p, double x, double y, double* phi, double* grad) {
    int k = 0;
    for (int td = 0; td <= p; ++td)
        for (int i = 0; i <= td; ++i, ++k) {
            const int j = td - i;
            if (phi) phi[k] = ipow(x, i) * ipow(y, j);
            if (grad) {
                grad[2 * k] = i == 0 ? 0.0 : i * ipow(x, i - 1) * ipow(y, j);
                grad[2 * k + 1] = j == 0 ? 0.0 : ipow(x, i) * j * ipow(y, j - 1);
            }
        }
}

// Jacobi P_n^(a,b) by the three-term recurrence (src/basis/dubiner.cpp:24-47)
static double jacobi(int n, double a, double b, double x) {
    if (n == 0) return 1.0;
    double p0 = 1.0, p1 = 0.5 * (a - b + (a + b + 2.0) * x);
    for (int k = 2; k <= n; ++k) {
        const double c = 2.0 * k + a + b;
        const double a1 = 2.0 * k * (k + a + b) * (c - 2.0);
        const double a2 = (c - 1.0) * (a * a - b * b);
        const double a3 = (c - 2.0) * (c - 1.0) * c;
        const double a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * c;
        const double p2 = ((a2 + a3 * x) * p1 - a4 * p0) / a1;
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

// DubinerBasis (src/basis/dubiner.cpp:55-168): collapsed coordinates r = 2 xi/(1-eta) - 1,
// s = 2 eta - 1, index order j outer / i inner, scaling 2 sqrt((2i+1)(i+j+1)).
static void dubiner(int p, double x, double y, double* phi, double* grad) {
    if (!(x >= 0 && y >= 0 && x + y <= 1)) {  // ReferenceTriangle::project_to_bounds
        x = std::max(0.0, std::min(1.0, x));
        y = std::max(0.0, std::min(1.0 - x, y));
    }
    const double om = 1.0 - y;
    const bool top = std::fabs(om) < 1e-14;
    const double r = top ? -1.0 : 2.0 * x / om - 1.0;
    const double s = 2.0 * y - 1.0;
    const double dr_dx = top ? 0.0 : 2.0 / om, dr_dy = top ? 0.0 : 2.0 * x / (om * om);
    const double ds_dy = top ? 0.0 : 2.0;
    int k = 0;
    for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p - j; ++i, ++k) {
            const double Pi = jacobi(i, 0.0, 0.0, r);
            const double Pj = jacobi(j, 2.0 * i + 1.0, 0.0, s);
            const double nrm = 2.0 * std::sqrt((2.0 * i + 1.0) * (i + j + 1.0));
            const double sc = std::pow(0.5 * (1.0 - s), (double)i);
            if (phi) phi[k] = nrm * Pi * Pj * sc;
            if (grad) {
                const double dPi = i > 0 ? 0.5 * (i + 1.0) * jacobi(i - 1, 1.0, 1.0, r) : 0.0;
                const double dPj = j > 0 ? 0.5 * (j + 2.0 * i + 2.0) * jacobi(j - 1, 2.0 * i + 2.0, 1.0, s) : 0.0;
                const double dsc = i > 0 ? -0.5 * i * std::pow(0.5 * (1.0 - s), (double)(i - 1)) : 0.0;
                const double dphi_dr = nrm * dPi * Pj * sc;
                const double dphi_ds = nrm * Pi * (dPj * sc + Pj * dsc);
                grad[2 * k] = dphi_dr * dr_dx;
                grad[2 * k + 1] = dphi_dr * dr_dy + dphi_ds * ds_dy;
            }
        }
}

// LegendreBasis (src/basis/legendre.cpp:27-110), quadrilaterals on [-1, 1]^2:
// phi_k = P_i(x) P_j(y), k = j (p+1) + i.  P_n by Bonnet's recurrence; P'_n from
// (x^2 - 1) P'_n = n (x P_n - P_{n-1}), with P'_n(+-1) = (+-1)^(n+1) n (n+1) / 2 at the ends.
static void legendre_1d(int p, double x, double* P, double* dP) {
    P[0] = 1.0;
    if (p >= 1) P[1] = x;
    for (int n = 2; n <= p; ++n) P[n] = ((2 * n - 1) * x * P[n - 1] - (n - 1) * P[n - 2]) / n;
    const bool end = std::fabs(std::fabs(x) - 1.0) < 1e-12;
    for (int n = 0; n <= p; ++n) {
        if (n == 0) dP[n] = 0.0;
        else if (end) dP[n] = 0.5 * n * (n + 1) * ((n % 2 == 0) ? 1.0 : -1.0) * (x > 0 ? 1.0 : -1.0);
        else dP[n] = n * (x * P[n] - P[n - 1]) / (x * x - 1.0);
    }
}

static void legendre(int p, double x, double y, double* phi, double* grad) {
    double Px[8], Py[8], dPx[8], dPy[8];
    legendre_1d(p, x, Px, dPx);
    legendre_1d(p, y, Py, dPy);
    int k = 0;
    for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p; ++i, ++k) {
            if (phi) phi[k] = Px[i] * Py[j];
            if (grad) {
                grad[2 * k] = dPx[i] * Py[j];
                grad[2 * k + 1] = Px[i] * dPy[j];
            }
        }
}

static void basis_eval(int basis, int p, double x, double y, double* phi, double* grad) {
    if (basis == DGX_BASIS_LEGENDRE) legendre(p, x, y, phi, grad);
    else if (basis == DGX_BASIS_DUBINER) dubiner(p, x, y, phi, grad);
    else monomial(p, x, y, phi, grad);
}

// DGSpace::map_face_quad_point (src/core/space.cpp:259-288): face f of a triangle (nf = 3)
// or a quadrilateral (nf = 4) at s in [-1, 1], running from vertex f to vertex f + 1.
static void face_point(int nf, int f, double s, double* xi) {
    if (nf == 4) {
        if (f == 0) { xi[0] = s; xi[1] = -1.0; }
        else if (f == 1) { xi[0] = 1.0; xi[1] = s; }
        else if (f == 2) { xi[0] = -s; xi[1] = 1.0; }
        else { xi[0] = -1.0; xi[1] = -s; }
        return;
    }
    const double t = 0.5 * (s + 1.0);
    if (f == 0) { xi[0] = t; xi[1] = 0.0; }
    else if (f == 1) { xi[0] = 1.0 - t; xi[1] = t; }
    else { xi[0] = 0.0; xi[1] = 1.0 - t; }
}

// ReferenceTriangle / ReferenceQuad::edge_vertices (src/reference/elements.cpp:27-38, 73-90):
// edge f runs from vertex f to vertex (f + 1) mod nv
static inline int edge_a(int f, int) { return f; }
static inline int edge_b(int f, int nv) { return (f + 1) % nv; }

static bool invert(int n, const double* A, double* X) {  // Gauss-Jordan, partial pivoting
    std::vector<double> M(A, A + n * n);
    for (int i = 0; i < n * n; ++i) X[i] = 0.0;
    for (int i = 0; i < n; ++i) X[i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(M[r * n + c]) > std::fabs(M[p * n + c])) p = r;
        if (M[p * n + c] == 0.0) return false;
        for (int k = 0; k < n; ++k) {
            std::swap(M[c * n + k], M[p * n + k]);
            std::swap(X[c * n + k], X[p * n + k]);
        }
        const double d = 1.0 / M[c * n + c];
        for (int k = 0; k < n; ++k) {
            M[c * n + k] *= d;
            X[c * n + k] *= d;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = M[r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                M[r * n + k] -= f * M[c * n + k];
                X[r * n + k] -= f * X[c * n + k];
            }
        }
    }
    return true;
}

// DGSpace ctor + precompute_basis_values (src/core/space.cpp:20-67, 230-257) and the
// reference mass matrix of TimeDependentWeakFormulation::compute_mass_integral
// (src/weak_forms/weak_formulation_base.cpp:198-217) divided by |J|.
//
// Quadrilaterals (basis DGX_BASIS_LEGENDRE): the tensor Gauss-Legendre rule with p+1 points
// per direction, point q = j (p+1) + i at (x_i, x_j) with weight w_i w_j
// (QuadratureFactory::gauss_legendre_quad, src/quadrature/factory.cpp:33-59).
int dgx::make_ops(int p, int basis, OpsHost& o) {
    std::memset(&o, 0, sizeof(o));
    const bool quad = basis == DGX_BASIS_LEGENDRE;
    const int order = 2 * p;
    if (p + 1 > DGX_GL_MAX_POINTS) return -1;
    if (quad ? p > MAX_P_QUAD : order > DGX_TRI_MAX_ORDER) return -1;
    o.p = p;
    o.nf = quad ? 4 : 3;
    o.np = quad ? n_basis_quad(p) : n_basis(p);
    o.nq = quad ? n_basis_quad(p) : dgx_tri_rule_npts[order];
    o.nfq = p + 1;
    if (!quad && o.nq != n_quad(p)) return -1;
    std::vector<double> qp(2 * o.nq), qw(o.nq);
    if (quad) {
        for (int j = 0; j <= p; ++j)
            for (int i = 0; i <= p; ++i) {
                const int q = j * (p + 1) + i;
                qp[2 * q] = dgx_gl_points[p][i];
                qp[2 * q + 1] = dgx_gl_points[p][j];
                qw[q] = dgx_gl_weights[p][i] * dgx_gl_weights[p][j];
            }
    } else {
        std::copy(dgx_tri_rule_points + 2 * dgx_tri_rule_offset[order],
                  dgx_tri_rule_points + 2 * (dgx_tri_rule_offset[order] + o.nq), qp.begin());
        std::copy(dgx_tri_rule_weights + dgx_tri_rule_offset[order],
                  dgx_tri_rule_weights + dgx_tri_rule_offset[order] + o.nq, qw.begin());
    }
    double phi[OPS_MAX_NP], g[2 * OPS_MAX_NP];
    for (int q = 0; q < o.nq; ++q) {
        o.qp[q][0] = qp[2 * q];
        o.qp[q][1] = qp[2 * q + 1];
        o.wq[q] = qw[q];
        basis_eval(basis, p, qp[2 * q], qp[2 * q + 1], phi, g);
        for (int i = 0; i < o.np; ++i) {
            o.phi[q][i] = phi[i];
            o.dr[q][i] = g[2 * i];
            o.ds[q][i] = g[2 * i + 1];
        }
    }
    for (int q = 0; q < o.nfq; ++q) {
        o.fp[q] = dgx_gl_points[p][q];
        o.wf[q] = dgx_gl_weights[p][q];
    }
    for (int f = 0; f < o.nf; ++f)
        for (int q = 0; q < o.nfq; ++q) {
            double xi[2];
            face_point(o.nf, f, o.fp[q], xi);
            o.fxi[f][q][0] = xi[0];
            o.fxi[f][q][1] = xi[1];
            basis_eval(basis, p, xi[0], xi[1], phi, g);
            for (int i = 0; i < o.np; ++i) {
                o.phif[f][q][i] = phi[i];
                o.drf[f][q][i] = g[2 * i];
                o.dsf[f][q][i] = g[2 * i + 1];
            }
        }
    std::vector<double> M(o.np * o.np, 0.0), Mi(o.np * o.np);
    for (int q = 0; q < o.nq; ++q)
        for (int i = 0; i < o.np; ++i)
            for (int j = 0; j < o.np; ++j) M[i * o.np + j] += o.wq[q] * (o.phi[q][i] * o.phi[q][j]);
    if (!invert(o.np, M.data(), Mi.data())) return -1;
    for (int i = 0; i < o.np; ++i)
        for (int j = 0; j < o.np; ++j) o.minv[i][j] = Mi[i * o.np + j];
    return 0;
}

// ------------------------------------------------------------------ mesh
struct BCDef {
    int type;
    double value[4];
};

struct dgx_mesh {
    int nvpe = 3;               // vertices (= faces) per element: 3 triangles, 4 quadrilaterals
    std::vector<double> verts;  // [nv][2]
    std::vector<int> elems;     // [ne][nvpe]
    std::map<std::string, int> tags;
    std::vector<int> nbr;       // [ne][nvpe][2] face_neighbors_
    std::vector<int> btag;      // [ne][nvpe] boundary_face_tags_ value, -1 when absent
    std::vector<int> ifaces;    // [n][5] L, R, fL, fR, reversed
    std::vector<int> bfaces;    // [n][3] elem, face, tag
    std::map<int, BCDef> bcs;   // by tag id
    int ne() const { return (int)elems.size() / nvpe; }
};

// GeometricMapping::compute_mapping (src/reference/mapping.cpp:22-50) for an affine
// triangle: J_T = dN^T V, A = inverse(J_T) by the 2x2 cofactor formula.
static bool affine_map(const double* V, double* A, double* det) {
    const double J00 = V[2] - V[0], J01 = V[3] - V[1];
    const double J10 = V[4] - V[0], J11 = V[5] - V[1];
    *det = J00 * J11 - J10 * J01;
    if (std::fabs(*det) < 1e-12) return false;
    const double inv = 1.0 / *det;
    A[0] = J11 * inv;
    A[2] = -J10 * inv;
    A[1] = -J01 * inv;
    A[3] = J00 * inv;
    return true;
}

// outward normal and length of face f of an element with nv vertices
// (DGSpace::compute_face_data, src/core/space.cpp:104-137)
static bool face_geom(const double* V, int nv, int f, double* n, double* len) {
    const double* v1 = V + 2 * edge_a(f, nv);
    const double* v2 = V + 2 * edge_b(f, nv);
    const double tx = v2[0] - v1[0], ty = v2[1] - v1[1];
    *len = std::sqrt(tx * tx + ty * ty);
    if (*len < 1e-14) return false;
    n[0] = ty / *len;
    n[1] = -tx / *len;
    double cx = 0.0, cy = 0.0;
    for (int k = 0; k < nv; ++k) {
        cx += V[2 * k];
        cy += V[2 * k + 1];
    }
    cx /= nv;
    cy /= nv;
    const double mx = 0.5 * (v1[0] + v2[0]), my = 0.5 * (v1[1] + v2[1]);
    if (n[0] * (mx - cx) + n[1] * (my - cy) < 0) {
        n[0] = -n[0];
        n[1] = -n[1];
    }
    return true;
}

static void elem_verts(const dgx_mesh* m, int e, double* V) {
    for (int k = 0; k < m->nvpe; ++k) {
        const int v = m->elems[(size_t)m->nvpe * e + k];
        V[2 * k] = m->verts[2 * v];
        V[2 * k + 1] = m->verts[2 * v + 1];
    }
}

// DGSpace::compute_face_permutation (src/core/space.cpp:173-228): reversed or not
static bool face_reversed(int nv, const double* VL, int fL, const double* VR, int fR) {
    const double* a1 = VL + 2 * edge_a(fL, nv);
    const double* b1 = VL + 2 * edge_b(fL, nv);
    const double* a2 = VR + 2 * edge_a(fR, nv);
    const double* b2 = VR + 2 * edge_b(fR, nv);
    auto dist = [](const double* p, const double* q) { return std::hypot(p[0] - q[0], p[1] - q[1]); };
    const double tol = 1e-10;
    const bool rev = dist(a1, b2) < tol && dist(b1, a2) < tol;
    const bool same = dist(a1, a2) < tol && dist(b1, b2) < tol;
    if (rev || same) return rev;
    const double t1x = b1[0] - a1[0], t1y = b1[1] - a1[1];
    const double t2x = b2[0] - a2[0], t2y = b2[1] - a2[1];
    return (t1x * t2x + t1y * t2y) / (std::hypot(t1x, t1y) * std::hypot(t2x, t2y)) < 0.0;
}

// DGMesh::build_precomputed_faces (src/core/mesh.cpp:404-480): interior faces in
// element-then-face order, de-duplicated by element pair; the rest are boundary faces.
static void rebuild_faces(dgx_mesh* m) {
    const int ne = m->ne(), K = m->nvpe;
    m->ifaces.clear();
    m->bfaces.clear();
    m->ifaces.reserve((size_t)ne * K / 2 * 5 + 16);
    double VL[8], VR[8];
    for (int L = 0; L < ne; ++L) {
        elem_verts(m, L, VL);
        const int* nb = &m->nbr[2 * (size_t)K * L];
        for (int fL = 0; fL < K; ++fL) {
            const int R = nb[2 * fL], fR = nb[2 * fL + 1];
            if (R >= 0) {
                // one face per element pair, at its first occurrence in element order (dgfem keys
                // its face set by the pair): met here when R >= L and no earlier face of L has R
                if (R < L) continue;
                bool earlier = false;
                for (int g = 0; g < fL; ++g) earlier |= nb[2 * g] == R;
                if (earlier) continue;
                elem_verts(m, R, VR);
                const int rec[5] = {L, R, fL, fR, face_reversed(K, VL, fL, VR, fR) ? 1 : 0};
                m->ifaces.insert(m->ifaces.end(), rec, rec + 5);
            } else {
                const int rec[3] = {L, fL, m->btag[(size_t)K * L + fL]};
                m->bfaces.insert(m->bfaces.end(), rec, rec + 3);
            }
        }
    }
}
// Face-slot pairing on the GPU (dgx_setup.cu) for meshes of at least this many face slots when a
// device is present; DGX_SETUP_ON_HOST=1 keeps it on the host, DGX_SETUP_ON_DEVICE=1 takes every
// mesh to the device.  Both give the same table.
static constexpr size_t DEVICE_PAIRING_MIN_SLOTS = 1 << 16;

static bool setup_on_device(size_t work) {
    const char* v = std::getenv("DGX_SETUP_ON_HOST");
    if (v && std::strcmp(v, "1") == 0) return false;
    const char* d = std::getenv("DGX_SETUP_ON_DEVICE");
    if (work < DEVICE_PAIRING_MIN_SLOTS && !(d && std::strcmp(d, "1") == 0)) return false;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return false;
    }
    return true;
}

static int build_connectivity(dgx_mesh* m, int nbe, const int* bedges) {
    const int ne = m->ne(), K = m->nvpe;
    const size_t ns = (size_t)ne * K;
    const uint64_t nv = (uint64_t)(m->verts.size() / 2);
    m->nbr.assign((size_t)ne * 2 * K, -1);
    if (setup_on_device(ns)) {
        if (device_face_pairs(ne, K, m->elems.data(), (long long)nv, m->nbr.data()))
            return fail(DGX_ERR_CUDA, std::string("face pairing on the device failed: ") + launch_error_text());
    } else {
        // face slots keyed by their vertex pair (min, max): a stable radix sort of the packed keys
        // keeps equal pairs in slot order (the first two slots of a pair become neighbours)
        std::vector<uint64_t> key(ns), key2(ns);
        std::vector<int> ord(ns), ord2(ns);
        for (int e = 0; e < ne; ++e)
            for (int f = 0; f < K; ++f) {
                const int v1 = m->elems[(size_t)K * e + f], v2 = m->elems[(size_t)K * e + (f + 1) % K];
                key[(size_t)K * e + f] = (uint64_t)std::min(v1, v2) * nv + (uint64_t)std::max(v1, v2);
                ord[(size_t)K * e + f] = K * e + f;
            }
        uint64_t kmax = 0;
        for (uint64_t k : key) kmax = std::max(kmax, k);
        for (int shift = 0; shift < 64 && (kmax >> shift) != 0; shift += 16) {
            std::vector<size_t> count(65537, 0);
            for (uint64_t k : key) ++count[((k >> shift) & 0xFFFF) + 1];
            for (int d = 0; d < 65536; ++d) count[d + 1] += count[d];
            for (size_t i = 0; i < ns; ++i) {
                const size_t pos = count[(key[i] >> shift) & 0xFFFF]++;
                key2[pos] = key[i];
                ord2[pos] = ord[i];
            }
            key.swap(key2);
            ord.swap(ord2);
        }
        for (size_t i = 0; i < ns;) {
            size_t j = i;
            while (j < ns && key[j] == key[i]) ++j;
            if (j - i >= 2) {  // the first two faces of a vertex pair become neighbours
                const int e1 = ord[i] / K, f1 = ord[i] % K, e2 = ord[i + 1] / K, f2 = ord[i + 1] % K;
                m->nbr[2 * ((size_t)K * e1 + f1)] = e2;
                m->nbr[2 * ((size_t)K * e1 + f1) + 1] = f2;
                m->nbr[2 * ((size_t)K * e2 + f2)] = e1;
                m->nbr[2 * ((size_t)K * e2 + f2) + 1] = f1;
            }
            i = j;
        }
    }
    m->btag.assign((size_t)ne * K, -1);
    if (nbe > 0) {
        // boundary_edges is a std::map keyed by tag: later tags override earlier ones
        std::vector<int> order(nbe);
        for (int k = 0; k < nbe; ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return bedges[3 * x] < bedges[3 * y]; });
        std::map<std::pair<int, int>, int> sig;
        for (int k : order) {
            const int v1 = bedges[3 * k + 1], v2 = bedges[3 * k + 2];
            sig[{std::min(v1, v2), std::max(v1, v2)}] = bedges[3 * k];
        }
        for (int e = 0; e < ne; ++e)
            for (int f = 0; f < K; ++f) {
                if (m->nbr[2 * ((size_t)K * e + f)] != -1) continue;
                const int v1 = m->elems[(size_t)K * e + f], v2 = m->elems[(size_t)K * e + (f + 1) % K];
                auto it = sig.find({std::min(v1, v2), std::max(v1, v2)});
                m->btag[(size_t)K * e + f] = it == sig.end() ? 0 : it->second;
            }
    }
    rebuild_faces(m);
    return DGX_OK;
}

extern "C" int dgx_mesh_create_nv(int nvpe, int nv, const double* verts, int ne, const int* elems, int n_tags,
                                  const char* const* tag_names, const int* tag_ids, int nbe, const int* bedges,
                                  dgx_mesh** out) {
    if (!out || nv < 0 || ne < 0 || (nv > 0 && !verts) || (ne > 0 && !elems) || (nbe > 0 && !bedges) ||
        (n_tags > 0 && (!tag_names || !tag_ids)))
        return fail(DGX_ERR_INVALID, "dgx_mesh_create: bad arguments");
    if (nvpe != 3 && nvpe != 4)  // DGMesh ctor (src/core/mesh.cpp:23-35)
        return fail(DGX_ERR_INVALID, "Unknown element type with " + std::to_string(nvpe) + " vertices");
    for (size_t i = 0; i < (size_t)nvpe * ne; ++i)
        if (elems[i] < 0 || elems[i] >= nv) return fail(DGX_ERR_RANGE, "element vertex index out of range");
    for (int k = 0; k < nbe; ++k)
        for (int c = 1; c < 3; ++c)
            if (bedges[3 * k + c] < 0) return fail(DGX_ERR_RANGE, "boundary edge vertex index out of range");
    auto* m = new dgx_mesh;
    m->nvpe = nvpe;
    m->verts.assign(verts, verts + 2 * (size_t)nv);
    m->elems.assign(elems, elems + (size_t)nvpe * ne);
    for (int t = 0; t < n_tags; ++t) m->tags[tag_names[t]] = tag_ids[t];
    build_connectivity(m, nbe, bedges);
    *out = m;
    return DGX_OK;
}

extern "C" int dgx_mesh_create(int nv, const double* verts, int ne, const int* elems, int n_tags,
                               const char* const* tag_names, const int* tag_ids, int nbe,
                               const int* bedges, dgx_mesh** out) {
    return dgx_mesh_create_nv(3, nv, verts, ne, elems, n_tags, tag_names, tag_ids, nbe, bedges, out);
}

extern "C" int dgx_mesh_vertices_per_element(const dgx_mesh* m, int* nvpe) {
    if (!m || !nvpe) return fail(DGX_ERR_INVALID, "null argument");
    *nvpe = m->nvpe;
    return DGX_OK;
}

// DGMesh::set_periodic_boundaries (src/core/mesh.cpp:482-588).  Like dgfem, the face list
// is rebuilt, which drops the boundary conditions set before.
extern "C" int dgx_mesh_set_periodic(dgx_mesh* m, const char* t1, const char* t2) {
    if (!m || !t1 || !t2) return fail(DGX_ERR_INVALID, "dgx_mesh_set_periodic: null argument");
    auto i1 = m->tags.find(t1), i2 = m->tags.find(t2);
    if (i1 == m->tags.end()) return fail(DGX_ERR_INVALID, std::string("Unknown boundary tag: ") + t1);
    if (i2 == m->tags.end()) return fail(DGX_ERR_INVALID, std::string("Unknown boundary tag: ") + t2);
    const int tag1 = i1->second, tag2 = i2->second;
    const std::string s1 = t1, s2 = t2;
    const bool match_y = s1 == "Left" || s1 == "Right" || s2 == "Left" || s2 == "Right";
    std::vector<int> f1, f2;
    for (size_t i = 0; i < m->btag.size(); ++i) {
        if (m->btag[i] < 0) continue;
        if (m->btag[i] == tag1) f1.push_back((int)i);
        else if (m->btag[i] == tag2) f2.push_back((int)i);
    }
    if (f1.empty() || f2.empty())
        return fail(DGX_ERR_RUNTIME, "Cannot set periodic boundaries: one or both boundaries have no faces");
    const int c = match_y ? 1 : 0, K = m->nvpe;
    auto center = [&](int slot) {
        const int e = slot / K, f = slot % K;
        const int a = m->elems[(size_t)K * e + f], b = m->elems[(size_t)K * e + (f + 1) % K];
        return 0.5 * (m->verts[2 * a + c] + m->verts[2 * b + c]);
    };
    // nearest transverse coordinate, first minimum wins: sort candidates once
    std::vector<std::pair<double, int>> cand(f2.size());
    for (size_t k = 0; k < f2.size(); ++k) cand[k] = {center(f2[k]), (int)k};
    std::sort(cand.begin(), cand.end());
    for (int s1f : f1) {
        const double x = center(s1f);
        auto it = std::lower_bound(cand.begin(), cand.end(), std::make_pair(x, -1));
        double best = std::numeric_limits<double>::max();
        int bi = -1;
        // examine the run of equal distances on both sides; ties go to the lowest index
        for (auto j = it; j != cand.end(); ++j) {
            const double d = std::fabs(x - j->first);
            if (d > best) break;
            if (d < best || (d == best && j->second < bi)) { best = d; bi = j->second; }
        }
        for (auto j = it; j != cand.begin();) {
            --j;
            const double d = std::fabs(x - j->first);
            if (d > best) break;
            if (d < best || (d == best && j->second < bi)) { best = d; bi = j->second; }
        }
        if (bi < 0) continue;
        const int e1 = s1f / K, l1 = s1f % K, e2 = f2[bi] / K, l2 = f2[bi] % K;
        m->nbr[2 * ((size_t)K * e1 + l1)] = e2;
        m->nbr[2 * ((size_t)K * e1 + l1) + 1] = l2;
        m->nbr[2 * ((size_t)K * e2 + l2)] = e1;
        m->nbr[2 * ((size_t)K * e2 + l2) + 1] = l1;
    }
    m->bcs.clear();
    rebuild_faces(m);
    return DGX_OK;
}

// Structured rectangle of nx x ny cells: two triangles per cell (nvpe = 3) or the cell
// itself (nvpe = 4), boundary tags Bottom=2 Right=3 Top=4 Left=5.
static int create_rectangle(int nvpe, int nx, int ny, double x0, double x1, double y0, double y1, int periodic,
                            dgx_mesh** out) {
    if (nx < 1 || ny < 1 || !out || !(x1 > x0) || !(y1 > y0))
        return fail(DGX_ERR_INVALID, "dgx_mesh_create_rectangle: bad arguments");
    const int nvx = nx + 1, nvy = ny + 1;
    std::vector<double> V((size_t)nvx * nvy * 2);
    for (int j = 0; j < nvy; ++j)
        for (int i = 0; i < nvx; ++i) {
            // x = i*((x1-x0)/nx) + x0 with the last point exactly x1 (numpy.linspace)
            const double sx = (x1 - x0) / nx, sy = (y1 - y0) / ny;
            V[2 * ((size_t)j * nvx + i)] = i == nx ? x1 : i * sx + x0;
            V[2 * ((size_t)j * nvx + i) + 1] = j == ny ? y1 : j * sy + y0;
        }
    auto vid = [&](int i, int j) { return j * nvx + i; };
    std::vector<int> E;
    E.reserve((size_t)nx * ny * 6);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int a = vid(i, j), b = vid(i + 1, j), c = vid(i + 1, j + 1), d = vid(i, j + 1);
            if (nvpe == 4) {
                E.insert(E.end(), {a, b, c, d});
            } else {
                E.insert(E.end(), {a, b, c, a, c, d});
            }
        }
    std::vector<int> B;
    for (int i = 0; i < nx; ++i) B.insert(B.end(), {2, vid(i, 0), vid(i + 1, 0)});
    for (int j = 0; j < ny; ++j) B.insert(B.end(), {3, vid(nx, j), vid(nx, j + 1)});
    for (int i = 0; i < nx; ++i) B.insert(B.end(), {4, vid(i, ny), vid(i + 1, ny)});
    for (int j = 0; j < ny; ++j) B.insert(B.end(), {5, vid(0, j), vid(0, j + 1)});
    const char* names[4] = {"Bottom", "Right", "Top", "Left"};
    const int ids[4] = {2, 3, 4, 5};
    int rc = dgx_mesh_create_nv(nvpe, nvx * nvy, V.data(), (int)(E.size() / nvpe), E.data(), 4, names, ids,
                                (int)B.size() / 3, B.data(), out);
    if (rc || !periodic) return rc;
    if ((rc = dgx_mesh_set_periodic(*out, "Left", "Right")) || (rc = dgx_mesh_set_periodic(*out, "Bottom", "Top"))) {
        dgx_mesh_destroy(*out);
        *out = nullptr;
    }
    return rc;
}

extern "C" int dgx_mesh_create_rectangle(int nx, int ny, double x0, double x1, double y0, double y1,
                                         int periodic, dgx_mesh** out) {
    return create_rectangle(3, nx, ny, x0, x1, y0, y1, periodic, out);
}

extern "C" int dgx_mesh_create_rectangle_quad(int nx, int ny, double x0, double x1, double y0, double y1,
                                              int periodic, dgx_mesh** out) {
    return create_rectangle(4, nx, ny, x0, x1, y0, y1, periodic, out);
}

extern "C" int dgx_mesh_set_bc(dgx_mesh* m, const char* tag, int type, const double* value4) {
    if (!m || !tag) return fail(DGX_ERR_INVALID, "dgx_mesh_set_bc: null argument");
    auto it = m->tags.find(tag);
    if (it == m->tags.end()) return fail(DGX_ERR_INVALID, std::string("Unknown boundary tag: ") + tag);
    if (type < DGX_BC_FAR_FIELD || type > DGX_BC_PERIODIC) return fail(DGX_ERR_INVALID, "unknown BC type");
    BCDef d;
    d.type = type;
    for (int v = 0; v < 4; ++v) d.value[v] = value4 ? value4[v] : 0.0;
    m->bcs[it->second] = d;
    return DGX_OK;
}

extern "C" int dgx_mesh_info(const dgx_mesh* m, int* ne, int* nif, int* nbf) {
    if (!m) return fail(DGX_ERR_INVALID, "null mesh");
    if (ne) *ne = m->ne();
    if (nif) *nif = (int)m->ifaces.size() / 5;
    if (nbf) *nbf = (int)m->bfaces.size() / 3;
    return DGX_OK;
}

extern "C" int dgx_mesh_interior_faces(const dgx_mesh* m, int* out5) {
    if (!m || !out5) return fail(DGX_ERR_INVALID, "null argument");
    std::copy(m->ifaces.begin(), m->ifaces.end(), out5);
    return DGX_OK;
}

extern "C" int dgx_mesh_boundary_faces(const dgx_mesh* m, int* out3) {
    if (!m || !out3) return fail(DGX_ERR_INVALID, "null argument");
    std::copy(m->bfaces.begin(), m->bfaces.end(), out3);
    return DGX_OK;
}

extern "C" int dgx_mesh_arrays(const dgx_mesh* m, int* nv, double* verts, int* elems) {
    if (!m) return fail(DGX_ERR_INVALID, "null mesh");
    if (nv) *nv = (int)m->verts.size() / 2;
    if (verts) std::copy(m->verts.begin(), m->verts.end(), verts);
    if (elems) std::copy(m->elems.begin(), m->elems.end(), elems);
    return DGX_OK;
}

extern "C" void dgx_mesh_destroy(dgx_mesh* m) { delete m; }

// ------------------------------------------------------------------ context

static StepArgs base_args(const dgx_ctx* c) {
    StepArgs a{};
    a.ne = c->ne;
    a.geom = c->d_geom;
    a.conn = c->d_conn;
    a.bc = c->d_bc;
    a.gamma = c->prm.gamma;
    a.mu = c->prm.mu;
    a.prandtl = c->prm.prandtl;
    a.sigma0 = c->prm.sigma0;
    a.order = c->prm.order;
    a.minv_diag = c->minv_diag;
    return a;
}

static int launch(const dgx_ctx* c, const StepArgs& a, cudaStream_t s) {
    const bool visc = c->prm.physics == DGX_NAVIER_STOKES;
    const int rc = c->nvpe == 4 ? launch_quad_element(c->prm.order, visc, c->prm.precision, a, c->d_qgeom,
                                                      c->d_qconn, c->ops, s)
                   : c->prm.precision == DGX_MIXED  ? launch_element_mixed(c->prm.order, visc, a, c->ops, s)
                   : c->prm.precision == DGX_DF64 ? launch_element_df64(c->prm.order, visc, a, c->ops, s)
                                                  : launch_element_fp64(c->prm.order, visc, a, c->ops, s);
    if (rc) return fail(DGX_ERR_CUDA, std::string("element kernel launch failed: ") +
                                          launch_error_text());
    return DGX_OK;
}

static void free_ctx(dgx_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    for (cudaGraphExec_t g : c->mgraph)
        if (g) cudaGraphExecDestroy(g);
    for (double* a : c->d_adj) cudaFree(a);
    cudaFree(c->d_kin);
    cudaFree(c->d_uhi[0]);
    cudaFree(c->d_uhi[1]);
    cudaFree(c->d_ulo);
    cudaFree(c->d_xq);
    cudaFree(c->d_d1);
    cudaFree(c->d_d2);
    cudaFree(c->d_tr[0]);
    cudaFree(c->d_tr[1]);
    cudaFree(c->d_tconn);
    cudaFree(c->d_ghost_bc);
    if (c->cap) cudaStreamDestroy(c->cap);
    if (c->host_out) cudaStreamDestroy(c->host_out);
    for (cudaEvent_t e : c->host_ev)
        if (e) cudaEventDestroy(e);
    cudaFree(c->d_geom);
    cudaFree(c->d_geomf);
    cudaFree(c->d_conn);
    cudaFree(c->d_qgeom);
    cudaFree(c->d_qconn);
    cudaFree(c->d_qgeomf);
    cudaFree(c->d_bc);
    cudaFree(c->d_u1);
    cudaFree(c->d_u2);
    cudaFree(c->d_hu);
    cudaFree(c->d_hr);
    cudaFree(c->d_mon);
    cudaFree(c->d_flag);
    cudaFree(c->d_status);
    delete c;
}

extern "C" void dgx_destroy(dgx_ctx* c) { free_ctx(c); }

// Face slots and boundary-condition slots shared by both element shapes: fn/fl hold every
// element's own outward normals and face lengths ([ne][NF][2], [ne][NF]).  With geom null only
// the connectivity and the slots are built (the device computes the geometry, dgx_setup.cu).
template <int NF, class Geom, class Conn>
static int face_slots(const dgx_mesh* m, const std::vector<double>& fn, const std::vector<double>& fl,
                      std::vector<Geom>* geom_or_null, std::vector<Conn>& conn, HostGeometry& g) {
    const int ne = m->ne();
    std::vector<BCSlot>& slots = g.slots;
    for (int e = 0; e < ne; ++e) {
        for (int f = 0; f < NF; ++f) conn[e].nbr[f] = NBR_SKIP;
        conn[e].flags = 0;
    }
    std::vector<char> taken((size_t)ne * NF, 0);
    auto take = [&](int e, int f) {
        if (taken[(size_t)NF * e + f]) return false;
        taken[(size_t)NF * e + f] = 1;
        return true;
    };
    const int nif = (int)m->ifaces.size() / 5;
    for (int k = 0; k < nif; ++k) {
        const int* F = &m->ifaces[5 * (size_t)k];
        const int L = F[0], R = F[1], fL = F[2], fR = F[3], rev = F[4];
        if (!take(L, fL) || !take(R, fR)) {
            return fail(DGX_ERR_RUNTIME, "unsupported mesh topology: an element face appears in two interior faces");
        }
        if (geom_or_null) {
            std::vector<Geom>& geom = *geom_or_null;
            const double* nL = &fn[2 * ((size_t)NF * L + fL)];
            const double hL = fl[(size_t)NF * L + fL];
            geom[L].n[fL][0] = nL[0];
            geom[L].n[fL][1] = nL[1];
            geom[L].h[fL] = hL;
            geom[R].n[fR][0] = -nL[0];
            geom[R].n[fR][1] = -nL[1];
            geom[R].h[fR] = hL;
        }
        conn[L].nbr[fL] = R;
        conn[L].flags |= (fR | (rev << 2) | (1 << 3)) << (4 * fL);
        conn[R].nbr[fR] = L;
        conn[R].flags |= (fL | (rev << 2)) << (4 * fR);
    }
    std::map<int, int> slot_of_tag;
    const int nbf = (int)m->bfaces.size() / 3;
    for (int k = 0; k < nbf; ++k) {
        const int e = m->bfaces[3 * (size_t)k], f = m->bfaces[3 * (size_t)k + 1], tag = m->bfaces[3 * (size_t)k + 2];
        if (geom_or_null) {
            (*geom_or_null)[e].n[f][0] = fn[2 * ((size_t)NF * e + f)];
            (*geom_or_null)[e].n[f][1] = fn[2 * ((size_t)NF * e + f) + 1];
            (*geom_or_null)[e].h[f] = fl[(size_t)NF * e + f];
        }
        auto it = m->bcs.find(tag);
        if (tag < 0 || it == m->bcs.end()) continue;  // no BC: dgfem skips the face
        if (it->second.type == DGX_BC_PERIODIC) {
            return fail(DGX_ERR_RUNTIME, "PERIODIC BC encountered in boundary_face_residual - periodic "
                                         "boundaries should be treated as interior faces");
        }
        auto si = slot_of_tag.find(tag);
        int slot;
        if (si == slot_of_tag.end()) {
            if ((int)slots.size() >= MAX_BC) {
                    return fail(DGX_ERR_RUNTIME, "too many boundary tags with conditions");
            }
            BCSlot b{};
            b.type = it->second.type;
            if (b.type == DGX_BC_SLIP_WALL) g.has_slip_wall = 1;
            for (int v = 0; v < 4; ++v) b.value[v] = it->second.value[v];
            slot = (int)slots.size();
            slots.push_back(b);
            slot_of_tag[tag] = slot;
        } else {
            slot = si->second;
        }
        conn[e].nbr[f] = -1 - slot;
        conn[e].flags |= (1 << 3) << (4 * f);
    }
    for (int e = 0; e < ne && !g.boundary; ++e)
        for (int f = 0; f < NF; ++f)
            if (conn[e].nbr[f] < 0) g.boundary = 1;
    if (slots.empty()) slots.push_back(BCSlot{});
    return DGX_OK;
}

// compute_max_cfl's h_elem (src/solver/compressible_solver_base.cpp:124-131): the shortest
// distance between two vertices of the element
static double shortest_vertex_distance(const double* V, int nv) {
    double h = std::numeric_limits<double>::max();
    for (int i = 0; i < nv; ++i)
        for (int j = i + 1; j < nv; ++j)
            h = std::min(h, std::sqrt((V[2 * i] - V[2 * j]) * (V[2 * i] - V[2 * j]) +
                                      (V[2 * i + 1] - V[2 * j + 1]) * (V[2 * i + 1] - V[2 * j + 1])));
    return h;
}

// Quadrilateral geometry: the bilinear map's derivative coefficients, faces and slots
// (DGSpace::compute_element_data / compute_face_data, src/core/space.cpp:69-171, with
// GeometricMapping::compute_mapping's singular-Jacobian check at the volume and face points).
static int build_geometry_quad(const dgx_mesh* m, const OpsHost& ops, HostGeometry& g) {
    const int ne = m->ne();
    g.qgeom.assign(ne, QuadGeom{});
    g.qconn.assign(ne, QuadConn{});
    std::vector<double> fn((size_t)ne * 8), fl((size_t)ne * 4);
    g.xq.resize((size_t)ne * ops.nq * 2);
    for (int e = 0; e < ne; ++e) {
        double V[8];
        elem_verts(m, e, V);
        QuadGeom& ge = g.qgeom[e];
        for (int c = 0; c < 2; ++c) {
            const double x0 = V[c], x1 = V[2 + c], x2 = V[4 + c], x3 = V[6 + c];
            double* j = c == 0 ? ge.jx : ge.jy;
            j[0] = 0.25 * ((x1 - x0) + (x2 - x3));
            j[1] = 0.25 * ((x3 - x0) + (x2 - x1));
            j[2] = 0.25 * ((x0 - x1) + (x2 - x3));
        }
        auto det_at = [&](double xi, double eta) {
            const double J00 = ge.jx[0] + ge.jx[2] * eta, J01 = ge.jy[0] + ge.jy[2] * eta;
            const double J10 = ge.jx[1] + ge.jx[2] * xi, J11 = ge.jy[1] + ge.jy[2] * xi;
            return J00 * J11 - J10 * J01;
        };
        for (int q = 0; q < ops.nq; ++q)
            if (std::fabs(det_at(ops.qp[q][0], ops.qp[q][1])) < 1e-12)
                return fail(DGX_ERR_RUNTIME, "Singular Jacobian matrix");
        for (int f = 0; f < 4; ++f)
            for (int q = 0; q < ops.nfq; ++q)
                if (std::fabs(det_at(ops.fxi[f][q][0], ops.fxi[f][q][1])) < 1e-12)
                    return fail(DGX_ERR_RUNTIME, "Singular Jacobian matrix");
        ge.hmin = shortest_vertex_distance(V, 4);
        for (int f = 0; f < 4; ++f)
            if (!face_geom(V, 4, f, &fn[8 * (size_t)e + 2 * f], &fl[4 * (size_t)e + f]))
                return fail(DGX_ERR_RUNTIME, "Degenerate edge detected");
        for (int q = 0; q < ops.nq; ++q) {  // map_to_physical: V^T N (ReferenceQuad shape functions)
            const double xi = ops.qp[q][0], eta = ops.qp[q][1];
            const double N[4] = {0.25 * (1.0 - xi) * (1.0 - eta), 0.25 * (1.0 + xi) * (1.0 - eta),
                                 0.25 * (1.0 + xi) * (1.0 + eta), 0.25 * (1.0 - xi) * (1.0 + eta)};
            double x = 0.0, y = 0.0;
            for (int k = 0; k < 4; ++k) {
                x += N[k] * V[2 * k];
                y += N[k] * V[2 * k + 1];
            }
            g.xq[((size_t)e * ops.nq + q) * 2] = x;
            g.xq[((size_t)e * ops.nq + q) * 2 + 1] = y;
        }
    }
    return face_slots<4>(m, fn, fl, &g.qgeom, g.qconn, g);
}

// Element geometry, face slots and boundary-condition slots of a mesh:
// DGSpace::compute_element_data / compute_face_data (src/core/space.cpp:69-171).
int dgx::build_geometry(const dgx_mesh* m, const OpsHost& ops, HostGeometry& g) {
    const int ne = m->ne();
    g.slots.clear();
    g.boundary = g.has_slip_wall = 0;
    if ((m->nvpe == 4) != (ops.nf == 4))
        return fail(DGX_ERR_INVALID, "the space's element type does not match the mesh's");
    if (m->nvpe == 4) return build_geometry_quad(m, ops, g);
    g.geom.assign(ne, ElemGeom{});
    g.conn.assign(ne, ElemConn{});
    std::vector<ElemGeom>& geom = g.geom;
    std::vector<double> fn((size_t)ne * 6), fl((size_t)ne * 3);
    g.xq.resize((size_t)ne * ops.nq * 2);
    for (int e = 0; e < ne; ++e) {
        double V[6], A[4], det;
        elem_verts(m, e, V);
        if (!affine_map(V, A, &det)) {
            return fail(DGX_ERR_RUNTIME, "Singular Jacobian matrix");
        }
        ElemGeom& ge = geom[e];
        std::memset(&ge, 0, sizeof(ge));
        for (int k = 0; k < 4; ++k) ge.A[k] = A[k];
        ge.detJ = std::fabs(det);
        ge.pad[0] = shortest_vertex_distance(V, 3);
        for (int f = 0; f < 3; ++f) {
            if (!face_geom(V, 3, f, &fn[6 * (size_t)e + 2 * f], &fl[3 * (size_t)e + f])) {
                    return fail(DGX_ERR_RUNTIME, "Degenerate edge detected");
            }
        }
        for (int q = 0; q < ops.nq; ++q) {  // map_to_physical: V^T N
            const double xi = ops.qp[q][0], eta = ops.qp[q][1];
            const double N0 = 1.0 - xi - eta;
            g.xq[((size_t)e * ops.nq + q) * 2] = N0 * V[0] + xi * V[2] + eta * V[4];
            g.xq[((size_t)e * ops.nq + q) * 2 + 1] = N0 * V[1] + xi * V[3] + eta * V[5];
        }
    }
    return face_slots<3>(m, fn, fl, &geom, g.conn, g);
}

// The connectivity and boundary slots of build_geometry without the geometry (dgx_create
// computes the geometry on the device).
int dgx::build_topology(const dgx_mesh* m, int nf, HostGeometry& g) {
    const int ne = m->ne();
    g.slots.clear();
    g.boundary = g.has_slip_wall = 0;
    if ((m->nvpe == 4) != (nf == 4))
        return fail(DGX_ERR_INVALID, "the space's element type does not match the mesh's");
    const std::vector<double> none;
    if (m->nvpe == 4) {
        g.qconn.assign(ne, QuadConn{});
        return face_slots<4, QuadGeom>(m, none, none, nullptr, g.qconn, g);
    }
    g.conn.assign(ne, ElemConn{});
    return face_slots<3, ElemGeom>(m, none, none, nullptr, g.conn, g);
}

ElemGeomF dgx::geom_to_f32(const ElemGeom& g, int instance) {
    ElemGeomF h;
    for (int k = 0; k < 4; ++k) h.A[k] = (float)g.A[k];
    h.detJ = (float)g.detJ;
    for (int f = 0; f < 3; ++f) {
        h.h[f] = (float)g.h[f];
        h.n[f][0] = (float)g.n[f][0];
        h.n[f][1] = (float)g.n[f][1];
    }
    h.hmin = (float)g.pad[0];
    std::memcpy(&h.pad, &instance, sizeof(float));  // batched solves: the element's instance
    return h;
}

int dgx::check_device(int* dev) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(DGX_ERR_CUDA, "no CUDA device: the dgx path has no CPU fallback");
    }
    CUDA_OK(cudaGetDevice(dev));
    cudaDeviceProp prop;
    CUDA_OK(cudaGetDeviceProperties(&prop, *dev));
    if (prop.major != 10 || prop.minor != 3)
        return fail(DGX_ERR_CUDA, "dgx kernels are built for sm_103a; this device is sm_" +
                                      std::to_string(prop.major) + std::to_string(prop.minor));
    return DGX_OK;
}

extern "C" int dgx_create(const dgx_mesh* m, const dgx_params* p, dgx_ctx** out) {
    if (!m || !p || !out) return fail(DGX_ERR_INVALID, "dgx_create: null argument");
    *out = nullptr;
    if (p->order < 1 || p->order > MAX_P)
        return fail(DGX_ERR_INVALID, "Element order must be between 1 and 4 for the GPU kernels");
    if (p->basis != DGX_BASIS_MONOMIAL && p->basis != DGX_BASIS_DUBINER && p->basis != DGX_BASIS_LEGENDRE)
        return fail(DGX_ERR_INVALID, "unknown basis");
    const bool quad = m->nvpe == 4;
    if (quad != (p->basis == DGX_BASIS_LEGENDRE))  // DGSpace::create_basis (src/core/space.cpp:307-319)
        return fail(DGX_ERR_INVALID, quad ? "quadrilateral meshes use the Legendre basis"
                                          : "the Legendre basis is for quadrilateral meshes");
    if (quad && p->order > MAX_P_QUAD)
        return fail(DGX_ERR_INVALID, "Element order must be between 1 and 4 for the quadrilateral GPU kernels");
    if (p->physics != DGX_EULER && p->physics != DGX_NAVIER_STOKES)
        return fail(DGX_ERR_INVALID, "unknown physics");
    if (p->precision != DGX_FP64 && p->precision != DGX_MIXED && p->precision != DGX_DF64)
        return fail(DGX_ERR_INVALID, "unknown precision");
    if (p->physics == DGX_NAVIER_STOKES) {  // NavierStokesWeakFormulation ctor checks (:22-33)
        if (p->mu <= 0.0) return fail(DGX_ERR_INVALID, "Dynamic viscosity must be positive for Navier-Stokes weak formulation");
        if (p->prandtl <= 0.0) return fail(DGX_ERR_INVALID, "Prandtl number must be positive for Navier-Stokes weak formulation");
        if (p->sigma0 <= 0.0) return fail(DGX_ERR_INVALID, "Penalty prefactor must be positive for Navier-Stokes weak formulation");
    }
    int dev = 0;
    if (int rc = check_device(&dev)) return rc;

    {
        const bool visc = p->physics == DGX_NAVIER_STOKES;
        int rc = quad                       ? configure_quad_element(p->order, visc, p->precision)
                 : p->precision == DGX_MIXED  ? configure_element_mixed(p->order, visc)
                 : p->precision == DGX_DF64 ? configure_element_df64(p->order, visc)
                                            : configure_element_fp64(p->order, visc);
        if (!rc && p->precision == DGX_MIXED && !visc && !quad) rc = configure_stage_tc(p->order);
        if (!rc && p->precision == DGX_MIXED && !visc && !quad) rc = configure_stage_trace(p->order);
        if (!rc && p->precision == DGX_MIXED && quad) rc = configure_quad_stage(p->order, visc);
        if (rc) return fail(DGX_ERR_CUDA, "could not configure the element kernel");
    }
    auto* c = new dgx_ctx;
    c->device = dev;
    c->prm = *p;
    c->nvpe = m->nvpe;
    if (make_ops(p->order, p->basis, c->ops)) {
        delete c;
        return fail(DGX_ERR_RUNTIME, "could not build reference operators");
    }
    {   // Dubiner: M_ref is diagonal up to round-off, so M_ref^-1 is applied as a scaling
        double dmax = 0.0, omax = 0.0;
        for (int i = 0; i < c->ops.np; ++i)
            for (int j = 0; j < c->ops.np; ++j)
                (i == j ? dmax : omax) = std::max(i == j ? dmax : omax, std::fabs(c->ops.minv[i][j]));
        c->minv_diag = omax <= 1e-12 * dmax ? 1 : 0;
    }
    const int ne = m->ne();
    c->ne = ne;
    c->np = c->ops.np;
    c->nq = c->ops.nq;
    c->nfq = c->ops.nfq;
    c->nstate = (size_t)ne * c->np * NV;

    // geometry on the device (dgx_setup.cu); DGX_SETUP_ON_HOST=1 builds it on the host instead
    // (the same records bit for bit)
    const char* hs = std::getenv("DGX_SETUP_ON_HOST");
    const bool host_setup = hs && std::strcmp(hs, "1") == 0;
    HostGeometry hg;
    if (int rc = host_setup ? build_geometry(m, c->ops, hg) : build_topology(m, c->ops.nf, hg)) {
        free_ctx(c);
        return rc;
    }
    std::vector<ElemGeom>& geom = hg.geom;
    std::vector<ElemConn>& conn = hg.conn;
    std::vector<BCSlot>& slots = hg.slots;
    c->xq = std::move(hg.xq);  // the host path's points; the device path fills it on first use
    c->boundary = hg.boundary;
    c->has_slip_wall = hg.has_slip_wall;

    auto alloc = [&](void** ptr, size_t bytes) {
        return cudaMalloc(ptr, bytes ? bytes : 16) == cudaSuccess;
    };
    const size_t sb = c->nstate * sizeof(double);
    // Face-trace form on a mesh with boundary faces: when every boundary face has a condition
    // (no skipped faces), boundary face k becomes an interior face to ghost block ne + k of the
    // trace buffers, which its owner fills with the ghost states of its traces; the stage then
    // runs the kernel without the boundary branch.
    const bool traces = p->precision == DGX_MIXED && !quad && p->physics == DGX_EULER;
    std::vector<ElemConn> tconn;
    std::vector<int> ghost_bc;
    if (traces && hg.boundary) {
        bool skipped = false;
        for (int e = 0; e < ne && !skipped; ++e)
            for (int f = 0; f < 3; ++f) skipped |= conn[e].nbr[f] == NBR_SKIP;
        if (!skipped) {
            tconn = conn;
            for (int e = 0; e < ne; ++e)
                for (int f = 0; f < 3; ++f)
                    if (conn[e].nbr[f] < 0) {
                        tconn[e].nbr[f] = ne + (int)ghost_bc.size();
                        tconn[e].flags &= ~(7 << (4 * f));  // the block's face 0, points in this face's order
                        ghost_bc.push_back(-1 - conn[e].nbr[f]);
                    }
        }
    }
    const size_t trace_blocks = (size_t)ne + ghost_bc.size();
    if ((quad ? !alloc((void**)&c->d_qgeom, sizeof(QuadGeom) * ne) || !alloc((void**)&c->d_qconn, sizeof(QuadConn) * ne)
              : !alloc((void**)&c->d_geom, sizeof(ElemGeom) * ne) || !alloc((void**)&c->d_conn, sizeof(ElemConn) * ne)) ||
        !alloc((void**)&c->d_bc, sizeof(BCSlot) * slots.size()) || !alloc((void**)&c->d_u1, sb) ||
        !alloc((void**)&c->d_xq, (size_t)ne * c->nq * 2 * sizeof(double)) ||
        (p->precision == DGX_MIXED && (quad ? !alloc((void**)&c->d_qgeomf, sizeof(QuadGeomF) * ne)
                                            : !alloc((void**)&c->d_geomf, sizeof(ElemGeomF) * ne))) ||
        !alloc((void**)&c->d_u2, sb) || !alloc((void**)&c->d_mon, 4 * sizeof(double)) ||
        !alloc((void**)&c->d_flag, sizeof(int)) || !alloc((void**)&c->d_status, sizeof(int)) ||
        (p->precision == DGX_MIXED &&
         (!alloc((void**)&c->d_uhi[0], c->nstate * sizeof(float)) ||
          !alloc((void**)&c->d_uhi[1], c->nstate * sizeof(float)) ||
          !alloc((void**)&c->d_ulo, c->nstate * sizeof(float)) ||
          !alloc((void**)&c->d_d1, c->nstate * sizeof(float)) ||
          !alloc((void**)&c->d_d2, c->nstate * sizeof(float)))) ||
        (p->precision == DGX_MIXED && !quad && p->physics == DGX_EULER &&
         (!alloc((void**)&c->d_tr[0], trace_blocks * trace_floats_per_element(p->order) * sizeof(float)) ||
          !alloc((void**)&c->d_tr[1], trace_blocks * trace_floats_per_element(p->order) * sizeof(float)))) ||
        (!ghost_bc.empty() && (!alloc((void**)&c->d_tconn, sizeof(ElemConn) * ne) ||
                               !alloc((void**)&c->d_ghost_bc, sizeof(int) * ghost_bc.size())))) {
        cudaGetLastError();
        free_ctx(c);
        return fail(DGX_ERR_CUDA, "cudaMalloc failed for the solver state");
    }
    bool geom_ok = true;
    if (host_setup) {  // upload the host-built records
        if (p->precision == DGX_MIXED && quad) {
            std::vector<QuadGeomF> gf(ne);
            for (int e = 0; e < ne; ++e) {
                const QuadGeom& g = hg.qgeom[e];
                QuadGeomF& h = gf[e];
                std::memset(&h, 0, sizeof(h));
                for (int k = 0; k < 3; ++k) {
                    h.jx[k] = (float)g.jx[k];
                    h.jy[k] = (float)g.jy[k];
                }
                for (int f = 0; f < 4; ++f) {
                    h.h[f] = (float)g.h[f];
                    h.n[f][0] = (float)g.n[f][0];
                    h.n[f][1] = (float)g.n[f][1];
                }
                h.hmin = (float)g.hmin;
            }
            geom_ok &= !ne || cudaMemcpy(c->d_qgeomf, gf.data(), sizeof(QuadGeomF) * ne, cudaMemcpyHostToDevice) ==
                                  cudaSuccess;
        }
        if (p->precision == DGX_MIXED && !quad) {
            std::vector<ElemGeomF> gf(ne);
            for (int e = 0; e < ne; ++e) gf[e] = geom_to_f32(geom[e], 0);
            geom_ok &= !ne || cudaMemcpy(c->d_geomf, gf.data(), sizeof(ElemGeomF) * ne, cudaMemcpyHostToDevice) ==
                                  cudaSuccess;
        }
        geom_ok &= !ne || (quad ? cudaMemcpy(c->d_qgeom, hg.qgeom.data(), sizeof(QuadGeom) * ne,
                                             cudaMemcpyHostToDevice) == cudaSuccess
                                : cudaMemcpy(c->d_geom, geom.data(), sizeof(ElemGeom) * ne, cudaMemcpyHostToDevice) ==
                                      cudaSuccess);
        geom_ok &= c->xq.empty() || cudaMemcpy(c->d_xq, c->xq.data(), c->xq.size() * sizeof(double),
                                               cudaMemcpyHostToDevice) == cudaSuccess;
    }
    geom_ok &= !ne || (quad ? cudaMemcpy(c->d_qconn, hg.qconn.data(), sizeof(QuadConn) * ne,
                                         cudaMemcpyHostToDevice) == cudaSuccess
                            : cudaMemcpy(c->d_conn, conn.data(), sizeof(ElemConn) * ne, cudaMemcpyHostToDevice) ==
                                  cudaSuccess);
    if (!host_setup && geom_ok && ne) {  // the geometry kernel, from the vertex and element arrays
        double* d_v = nullptr;
        int *d_e = nullptr, *d_err = nullptr;
        int err = 0;
        const bool ok = cudaMalloc((void**)&d_v, m->verts.size() * sizeof(double)) == cudaSuccess &&
                        cudaMalloc((void**)&d_e, m->elems.size() * sizeof(int)) == cudaSuccess &&
                        cudaMalloc((void**)&d_err, sizeof(int)) == cudaSuccess &&
                        cudaMemcpy(d_v, m->verts.data(), m->verts.size() * sizeof(double), cudaMemcpyHostToDevice) ==
                            cudaSuccess &&
                        cudaMemcpy(d_e, m->elems.data(), m->elems.size() * sizeof(int), cudaMemcpyHostToDevice) ==
                            cudaSuccess &&
                        cudaMemset(d_err, 0, sizeof(int)) == cudaSuccess &&
                        launch_device_geometry(ne, m->nvpe, c->ops, d_v, d_e,
                                               quad ? (const void*)c->d_qconn : (const void*)c->d_conn,
                                               quad ? (void*)c->d_qgeom : (void*)c->d_geom,
                                               quad ? (void*)c->d_qgeomf : (void*)c->d_geomf, c->d_xq, d_err,
                                               nullptr) == 0 &&
                        cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
        cudaFree(d_v);
        cudaFree(d_e);
        cudaFree(d_err);
        if (!ok) {
            cudaGetLastError();
            free_ctx(c);
            return fail(DGX_ERR_CUDA, "geometry set-up on the device failed");
        }
        if (err & 1) {
            free_ctx(c);
            return fail(DGX_ERR_RUNTIME, "Singular Jacobian matrix");
        }
        if (err & 2) {
            free_ctx(c);
            return fail(DGX_ERR_RUNTIME, "Degenerate edge detected");
        }
    }
    if (cudaMemset(c->d_status, 0, sizeof(int)) != cudaSuccess || !geom_ok ||
        (c->d_d1 && cudaMemset(c->d_d1, 0, c->nstate * sizeof(float)) != cudaSuccess) ||
        cudaMemcpy(c->d_bc, slots.data(), sizeof(BCSlot) * slots.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        (c->d_tconn &&
         (cudaMemcpy(c->d_tconn, tconn.data(), sizeof(ElemConn) * ne, cudaMemcpyHostToDevice) != cudaSuccess ||
          cudaMemcpy(c->d_ghost_bc, ghost_bc.data(), sizeof(int) * ghost_bc.size(), cudaMemcpyHostToDevice) !=
              cudaSuccess)) ||
        cudaStreamCreateWithFlags(&c->cap, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        free_ctx(c);
        return fail(DGX_ERR_CUDA, "device upload failed");
    }
    // the allocation-free stepping entry point's scratch array and kernels, loaded here so
    // that dgx_rk3_step_static itself allocates nothing (triangle meshes only)
    if (!quad) {
        if (int rc = static_scratch_setup(dev)) {
            free_ctx(c);
            return rc;
        }
    }
    *out = c;
    return DGX_OK;
}

extern "C" int dgx_launch_shape(const dgx_ctx* c, int* grid, int* tiles, int* form) {
    if (!c) return fail(DGX_ERR_INVALID, "null context");
    if (grid) *grid = c->stage_grid & ~STAGE_FLAGS;
    if (form)
        *form = (c->stage_grid & STAGE_TC)      ? 1
                : (c->stage_grid & STAGE_PIPE)  ? 3
                : (c->stage_grid & STAGE_TRACE) ? 2
                                                : 0;
    if (tiles) *tiles = (c->ne + TILE - 1) / TILE;
    return DGX_OK;
}

extern "C" int dgx_stage_tile(const dgx_ctx* c, int* elements, int* nbr_shared) {
    if (!c || !elements) return fail(DGX_ERR_INVALID, "null argument");
    *elements = c->stage_grid == 0             ? 0
                : (c->stage_grid & STAGE_T64) ? 64
                : (c->stage_grid & STAGE_T32) ? 32
                                              : TILE;
    if (nbr_shared) *nbr_shared = (c->stage_grid & STAGE_NBS) ? 1 : 0;
    return DGX_OK;
}

extern "C" int dgx_info(const dgx_ctx* c, int* ne, int* np, int* nq, int* nfq) {
    if (!c) return fail(DGX_ERR_INVALID, "null context");
    if (ne) *ne = c->ne;
    if (np) *np = c->np;
    if (nq) *nq = c->nq;
    if (nfq) *nfq = c->nfq;
    return DGX_OK;
}

extern "C" int dgx_residual(dgx_ctx* c, const double* u, double* r, void* stream) {
    if (!c || (c->ne && (!u || !r))) return fail(DGX_ERR_INVALID, "dgx_residual: null argument");
    if (u == r) return fail(DGX_ERR_INVALID, "dgx_residual: r may not alias u");
    StepArgs a = base_args(c);
    a.mode = MODE_RESIDUAL;
    a.u = u;
    a.out = r;
    return launch(c, a, (cudaStream_t)stream);
}

extern "C" int dgx_rhs(dgx_ctx* c, const double* u, double* du, void* stream) {
    if (!c || (c->ne && (!u || !du))) return fail(DGX_ERR_INVALID, "dgx_rhs: null argument");
    if (u == du) return fail(DGX_ERR_INVALID, "dgx_rhs: du may not alias u");
    StepArgs a = base_args(c);
    a.mode = MODE_RHS;
    a.u = u;
    a.out = du;
    return launch(c, a, (cudaStream_t)stream);
}

extern "C" int dgx_apply_mass_inv(dgx_ctx* c, const double* in, double* out, void* stream) {
    if (!c || (c->ne && (!in || !out))) return fail(DGX_ERR_INVALID, "dgx_apply_mass_inv: null argument");
    const int rc = c->nvpe == 4 ? launch_quad_mass_inv(c->ne, c->prm.order, c->ops, c->d_qgeom, in, out, (cudaStream_t)stream)
                                : launch_mass_inv(c->ne, c->prm.order, c->ops, c->d_geom, in, out, (cudaStream_t)stream);
    if (rc) return fail(DGX_ERR_CUDA, "mass inverse launch failed");
    return DGX_OK;
}

// The three SSP-RK3 stages (time_stepping.hpp:39-55):
//   u1 = u + dt L(u);  u2 = 3/4 u + 1/4 (u1 + dt L(u1));  u <- 1/3 u + 2/3 (u2 + dt L(u2))
// The last stage writes u in place: each element reads only its own u^n entries there.
static int enqueue_rk3(dgx_ctx* c, double* u, double dt, cudaStream_t s) {
    StepArgs a = base_args(c);
    a.mode = MODE_STAGE;
    a.status = c->d_status;
    a.dt = dt;
    a.u = u; a.un = nullptr; a.out = c->d_u1; a.a = 0.0; a.b = 1.0;
    int rc = launch(c, a, s);
    if (rc) return rc;
    a.u = c->d_u1; a.un = u; a.out = c->d_u2; a.a = 0.75; a.b = 0.25;
    if ((rc = launch(c, a, s))) return rc;
    a.u = c->d_u2; a.un = u; a.out = u; a.a = 1.0 / 3.0; a.b = 2.0 / 3.0;
    return launch(c, a, s);
}

extern "C" int dgx_rk3_stage(dgx_ctx* c, const double* u_n, const double* u_s, double* out, double dt, int stage,
                             void* stream) {
    if (!c || stage < 1 || stage > 3 || (c->ne && (!u_n || !u_s || !out)) || (c->ne && out == u_s))
        return fail(DGX_ERR_INVALID, "dgx_rk3_stage: bad argument");
    if (c->prm.precision == DGX_MIXED)
        return fail(DGX_ERR_INVALID, "dgx_rk3_stage: FP64 and double-float contexts only");
    if (c->ne == 0) return DGX_OK;
    static const double A[3] = {0.0, 0.75, 1.0 / 3.0}, B[3] = {1.0, 0.25, 2.0 / 3.0};
    StepArgs a = base_args(c);
    a.mode = MODE_STAGE;
    a.status = c->d_status;
    a.dt = dt;
    a.u = u_s;
    a.un = stage == 1 ? nullptr : u_n;
    a.out = out;
    a.a = A[stage - 1];
    a.b = B[stage - 1];
    return launch(c, a, (cudaStream_t)stream);
}

// Mixed precision: the three stages of one step, reading the FP32 copy uhi[src] of u^n
// and writing the FP32 copy of u^{n+1} to uhi[1 - src] (see StageArgs).
static StageArgs mixed_stage_args(const dgx_ctx* c, double* u, double dt, int src) {
    StageArgs a{};
    a.ne = c->ne;
    a.geom = c->d_geomf;
    a.conn = c->d_conn;
    a.qgeom = c->d_qgeomf;  // quadrilaterals (the triangle records are then null)
    a.qconn = c->d_qconn;
    a.bc = c->d_bc;
    a.dt = (float)dt;
    a.gamma = (float)c->prm.gamma;
    a.mu = (float)c->prm.mu;
    a.kappa = c->prm.physics == DGX_NAVIER_STOKES
                  ? (float)(c->prm.mu * c->prm.gamma / (c->prm.prandtl * (c->prm.gamma - 1.0)))
                  : 0.0f;
    a.sigma0 = (float)c->prm.sigma0;
    a.boundary = c->boundary;
    a.uhi = c->d_uhi[src];
    a.u64 = u;
    a.ulo = c->d_ulo;
    a.uhi_out = c->d_uhi[1 - src];
    a.grid = c->stage_grid;
    a.status = c->d_status;
    a.tconn = c->d_tconn;
    a.ghost_bc = c->d_ghost_bc;
    return a;
}

// Face-trace form: the stages of a step that starts from uhi[q] read the traces in d_tr[q],
// d_tr[1-q], d_tr[q] and write d_tr[1-q], d_tr[q], d_tr[1-q]: the next step starts from
// uhi[1-q] with its traces in d_tr[1-q].  kind: the step's place in its call (StepKind).
static void mixed_step_args(const dgx_ctx* c, double* u, double dt, int src, StageArgs st[3],
                            StepKind kind = STEP_ONLY) {
    StageArgs a = mixed_stage_args(c, u, dt, src);
    set_step_kind(a, kind);
    float* const t0 = c->d_tr[src];
    float* const t1 = c->d_tr[1 - src];
    st[0] = a; st[0].stage = 1; st[0].din = nullptr;   st[0].dout = c->d_d1;  st[0].tin = t0; st[0].tout = t1;
    st[1] = a; st[1].stage = 2; st[1].din = c->d_d1;   st[1].dout = c->d_d2;  st[1].tin = t1; st[1].tout = t0;
    st[2] = a; st[2].stage = 3; st[2].din = c->d_d2;   st[2].dout = nullptr;  st[2].tin = t0; st[2].tout = t1;
}

static int launch_stage(const dgx_ctx* c, const StageArgs& a, cudaStream_t s) {
    if (launch_stage_mixed(c->prm.order, c->prm.physics == DGX_NAVIER_STOKES, a, c->ops, s))
        return fail(DGX_ERR_CUDA, std::string("stage kernel launch failed: ") + launch_error_text());
    return DGX_OK;
}

static int enqueue_rk3_mixed(dgx_ctx* c, double* u, double dt, int src, StepKind kind, cudaStream_t s) {
    StageArgs st[3];
    mixed_step_args(c, u, dt, src, st, kind);
    for (const StageArgs& t : st)
        if (int rc = launch_stage(c, t, s)) return rc;
    return DGX_OK;
}

static int capture(dgx_ctx* c, cudaGraphExec_t* out, const std::function<int(cudaStream_t)>& body) {
    cudaGraph_t g;
    CUDA_OK(cudaStreamBeginCapture(c->cap, cudaStreamCaptureModeThreadLocal));
    const int rc = body(c->cap);
    const cudaError_t ec = cudaStreamEndCapture(c->cap, &g);
    if (rc) return rc;
    if (ec != cudaSuccess) return fail(DGX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        *out = nullptr;
        return fail(DGX_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    return DGX_OK;
}

static void destroy_graphs(dgx_ctx* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    for (cudaGraphExec_t& g : c->mgraph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

// Mixed precision, before the first step of a call: the FP32 copy of the caller's state
// (read by the first stage), the face traces of that state (trace form), and the stage
// kernel's launch shape and form (timed the first time).
static int mixed_prologue(dgx_ctx* c, double* u, double dt, cudaStream_t s) {
    if (launch_f64_to_f32(c->nstate, u, c->d_uhi[0], s))
        return fail(DGX_ERR_CUDA, std::string("conversion launch failed: ") + launch_error_text());
    // face-trace and tensor-core forms: the traces of the state the first step starts from
    // (uhi[0] -> d_tr[0]), each form with its own operations
    auto init_traces = [&](bool tc) {
        StageArgs t = mixed_stage_args(c, u, dt, 0);
        t.tout = c->d_tr[0];
        const int rc = tc ? launch_tc_trace_init(c->prm.order, t, c->ops, c->stage_grid & ~STAGE_TC, s)
                          : launch_trace_init(c->prm.order, t, c->ops, s);
        return rc ? fail(DGX_ERR_CUDA, std::string("trace launch failed: ") + launch_error_text()) : DGX_OK;
    };
    if (c->stage_grid == 0 && c->nvpe == 4) c->stage_grid = (c->ne + TILE - 1) / TILE;  // one launch shape
    if (c->stage_grid == 0) {
        // launch shape and form of the stage kernel
        const StageArgs a = mixed_stage_args(c, u, dt, 0);
        const bool visc = c->prm.physics == DGX_NAVIER_STOKES;
        // candidates: the neighbour-row form at each grid; for Euler the face-trace form at each
        // grid and at 64- and 32-element tiles, its pipelined persistent kernel at 2 and 3 CTAs per
        // SM (meshes whose faces are all interior or ghost faces) and the tensor-core form (orders
        // 1-3, the same meshes) at one CTA per SM.  DGX_STAGE_KERNEL=rows / =trace / =pipe / =tc
        // keeps one form (=trace: both trace kernels, every tile size), =trace64 / =trace32 /
        // =trace32s one tile size of the face-trace kernel.
        const int ntiles = (c->ne + TILE - 1) / TILE;
        const char* mode = std::getenv("DGX_STAGE_KERNEL");
        const bool only_tc = mode && std::strcmp(mode, "tc") == 0;
        const bool only_pipe = mode && std::strcmp(mode, "pipe") == 0;
        const bool only_trace = (mode && std::strcmp(mode, "trace") == 0) || only_pipe;
        const bool only_rows = mode && std::strcmp(mode, "rows") == 0;
        const bool tc_ok = !visc && c->d_tr[0] && stage_tc_supported(c->prm.order) && (!c->boundary || c->d_tconn);
        const bool pipe_ok = !visc && c->d_tr[0] && (!c->boundary || c->d_tconn);
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
        std::vector<int> cands;
        const std::vector<int> grids = grid_candidates(ntiles);
        if (visc || (!only_tc && !only_trace) || (only_tc && !tc_ok) || (only_pipe && !pipe_ok))
            cands = grids;  // the neighbour-row form
        if (!visc && c->d_tr[0] && !only_tc && !only_rows) {
            if (!only_pipe) {
                for (int g : grids) cands.push_back(STAGE_TRACE | g);
                // 64- and 32-element tiles, one CTA per tile
                cands.push_back(STAGE_TRACE | STAGE_T64 | ntiles);
                cands.push_back(STAGE_TRACE | STAGE_T32 | ntiles);
                if (pipe_ok) cands.push_back(STAGE_TRACE | STAGE_T32 | STAGE_NBS | ntiles);
            }
            if (pipe_ok)
                for (int k = 2; k <= 3; ++k) cands.push_back(STAGE_TRACE | STAGE_PIPE | std::min(ntiles, sms * k));
        }
        if (tc_ok && !only_trace && !only_rows) {
            cands.push_back(STAGE_TC | std::min(ntiles, sms * stage_tc_ctas_per_sm(c->prm.order)));
        }
        // =trace64 / =trace32: the face-trace kernel at that tile size only; =trace32s: at 32-element
        // tiles with the neighbours' trace blocks through shared memory where every face is an
        // interior or ghost face (else as =trace32)
        const bool only_t64 = mode && std::strcmp(mode, "trace64") == 0;
        const bool only_t32s = mode && std::strcmp(mode, "trace32s") == 0;
        if (!visc && c->d_tr[0] && (only_t64 || only_t32s || (mode && std::strcmp(mode, "trace32") == 0)))
            cands = {STAGE_TRACE | (only_t64 ? STAGE_T64 : STAGE_T32) | (only_t32s && pipe_ok ? STAGE_NBS : 0) | ntiles};
        // the traces the timed launches read (their rounding does not matter for the timing)
        if (c->d_tr[0])
            if (int rc = init_traces(false)) return rc;
        // the forms on offer depend on the boundary faces: none, all with ghost blocks, or some
        // without a condition (no ghost blocks: neither the pipelined nor the tensor-core form)
        const std::string key = "stage p" + std::to_string(c->prm.order) + (visc ? " ns" : " euler") +
                                (c->d_tconn ? " ghost" : c->boundary ? " bnd" : "") + " ne" + std::to_string(c->ne) +
                                " " + (mode ? mode : "");
        // timed as stage 2 (state uhi + d1, the increment zeroed at creation), which reads the
        // increment as stages 2 and 3 do; it writes only scratch (d2 and the traces in d_tr[1])
        int rc = tune_grid(key, cands, [&](int grid, cudaStream_t ts) {
            StageArgs t = a;
            t.stage = 2;
            t.din = c->d_d1;
            t.dout = c->d_d2;
            t.tin = c->d_tr[0];
            t.tout = c->d_tr[1];
            t.grid = grid;
            return launch_stage_mixed(c->prm.order, visc, t, c->ops, ts);
        }, s, &c->stage_grid);
        if (rc) return rc;
        destroy_graphs(c);
    }
    if (c->d_tr[0] && (c->stage_grid & (STAGE_TRACE | STAGE_TC)))
        if (int rc = init_traces((c->stage_grid & STAGE_TC) != 0)) return rc;
    return DGX_OK;
}

// dgx_rk3_step; with all_but_last (mixed precision, n_steps >= 2) the call's last step is left
// to the caller (dgx_rk3_step_host), which runs it as STEP_LAST from uhi[(n_steps - 1) & 1].
static int rk3_step_impl(dgx_ctx* c, double* u, double dt, int n_steps, cudaStream_t s, bool all_but_last) {
    const bool mixed = c->prm.precision == DGX_MIXED;
    if (mixed && (reinterpret_cast<uintptr_t>(u) & 15))  // the stage kernels move the state in 16-byte pieces
        return fail(DGX_ERR_INVALID, "dgx_rk3_step: a mixed-precision state must be 16-byte aligned");
    if (mixed)
        if (int rc = mixed_prologue(c, u, dt, s)) return rc;
    if (c->graph_u != u || c->graph_dt != dt) {
        destroy_graphs(c);
        c->graph_u = u;
        c->graph_dt = dt;
    }
    if (!mixed) {
        if (!c->graph)
            if (int rc = capture(c, &c->graph, [&](cudaStream_t cs) { return enqueue_rk3(c, u, dt, cs); })) return rc;
        for (int i = 0; i < n_steps; ++i) CUDA_OK(cudaGraphLaunch(c->graph, s));
        return DGX_OK;
    }
    // the call's steps as replays of the StepGraph graphs, each captured on first use
    return for_step_graphs(n_steps, [&](int g) {
        if (all_but_last && (g == G_LAST0 || g == G_LAST1)) return (int)DGX_OK;
        if (!c->mgraph[g]) {
            GraphStep gs[2];
            const int ns = graph_steps(g, gs);
            if (int rc = capture(c, &c->mgraph[g], [&](cudaStream_t cs) {
                    for (int k = 0; k < ns; ++k)
                        if (int r = enqueue_rk3_mixed(c, u, dt, gs[k].src, gs[k].kind, cs)) return r;
                    return (int)DGX_OK;
                }))
                return rc;
        }
        CUDA_OK(cudaGraphLaunch(c->mgraph[g], s));
        return (int)DGX_OK;
    });
}

extern "C" int dgx_rk3_step(dgx_ctx* c, double* u, double dt, int n_steps, void* stream) {
    if (!c || (c->ne && !u) || n_steps < 0) return fail(DGX_ERR_INVALID, "dgx_rk3_step: bad argument");
    if (c->ne == 0 || n_steps == 0) return DGX_OK;
    return rk3_step_impl(c, u, dt, n_steps, (cudaStream_t)stream, false);
}

static int monitor(dgx_ctx* c, const double* u, double dt, cudaStream_t s) {
    return c->nvpe == 4 ? launch_quad_monitor(c->ne, c->prm.order, c->ops, c->d_qgeom, u, dt, c->prm.gamma, c->d_mon, s)
                        : launch_monitor(c->ne, c->prm.order, c->ops, c->d_geom, u, dt, c->prm.gamma, c->d_mon, s);
}

extern "C" int dgx_max_cfl(dgx_ctx* c, const double* u, double dt, double* cfl, void* stream) {
    if (!c || !cfl || (c->ne && !u)) return fail(DGX_ERR_INVALID, "dgx_max_cfl: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (monitor(c, u, dt, s)) return fail(DGX_ERR_CUDA, "monitor launch failed");
    double h[4];
    CUDA_OK(cudaMemcpyAsync(h, c->d_mon, sizeof(h), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    *cfl = h[3] > 0.0 ? INFINITY : h[0];
    return DGX_OK;
}

extern "C" int dgx_density_range(dgx_ctx* c, const double* u, double* rmin, double* rmax, void* stream) {
    if (!c || !rmin || !rmax || (c->ne && !u)) return fail(DGX_ERR_INVALID, "dgx_density_range: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (monitor(c, u, 0.0, s)) return fail(DGX_ERR_CUDA, "monitor launch failed");
    double h[4];
    CUDA_OK(cudaMemcpyAsync(h, c->d_mon, sizeof(h), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    if (!std::isfinite(h[1]) || !std::isfinite(h[2])) {
        *rmin = *rmax = NAN;
    } else {
        *rmin = h[1];
        *rmax = h[2];
    }
    return DGX_OK;
}

extern "C" int dgx_has_nan(dgx_ctx* c, const double* u, int* has_nan, void* stream) {
    if (!c || !has_nan || (c->ne && !u)) return fail(DGX_ERR_INVALID, "dgx_has_nan: null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (launch_has_nan(c->nstate, u, c->d_flag, s)) return fail(DGX_ERR_CUDA, "nan scan launch failed");
    int f = 0;
    CUDA_OK(cudaMemcpyAsync(&f, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    *has_nan = f ? 1 : 0;
    return DGX_OK;
}

extern "C" int dgx_step_status(dgx_ctx* c, int* nonfinite, void* stream) {
    if (!c) return fail(DGX_ERR_INVALID, "null context");
    cudaStream_t s = (cudaStream_t)stream;
    int f = 0;
    CUDA_OK(cudaMemcpyAsync(&f, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    CUDA_OK(cudaStreamSynchronize(s));
    if (nonfinite) *nonfinite = f & 1;
    if (f & 2)
        return fail(DGX_ERR_TIMEOUT, "a bounded wait inside a stage kernel (tensor-core or pipelined trace form) "
                                     "gave up; the step's results are not valid");
    return (f & 1) ? fail(DGX_ERR_NONFINITE, "an SSP-RK3 step produced a non-finite value") : DGX_OK;
}

extern "C" int dgx_quad_points(const dgx_ctx* c, double* xq) {
    if (!c || !xq) return fail(DGX_ERR_INVALID, "dgx_quad_points: null argument");
    const size_t n = (size_t)c->ne * c->nq * 2;
    if (c->xq.size() != n) {  // the device-built points, copied once
        c->xq.resize(n);
        if (n) CUDA_OK(cudaMemcpy(c->xq.data(), c->d_xq, n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    std::copy(c->xq.begin(), c->xq.end(), xq);
    return DGX_OK;
}

extern "C" int dgx_quad_points_device(const dgx_ctx* c, double* xq, void* stream) {
    if (!c || (c->ne && !xq)) return fail(DGX_ERR_INVALID, "dgx_quad_points_device: bad argument");
    const size_t n = (size_t)c->ne * c->nq * 2;
    if (n) CUDA_OK(cudaMemcpyAsync(xq, c->d_xq, n * sizeof(double), cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return DGX_OK;
}

extern "C" int dgx_project(dgx_ctx* c, const double* uq, double* u, void* stream) {
    if (!c || (c->ne && (!uq || !u))) return fail(DGX_ERR_INVALID, "dgx_project: null argument");
    const int rc = c->nvpe == 4 ? launch_quad_project(c->ne, c->prm.order, c->ops, c->d_qgeom, uq, u, (cudaStream_t)stream)
                                : launch_project(c->ne, c->prm.order, c->ops, c->d_geom, uq, u, (cudaStream_t)stream);
    if (rc) return fail(DGX_ERR_CUDA, "projection launch failed");
    return DGX_OK;
}

extern "C" int dgx_eval_points(dgx_ctx* c, int n_points, const double* ref_xy, const double* u, double* out,
                               void* stream) {
    if (!c || n_points < 0 || (n_points && !ref_xy) || (c->ne && n_points && (!u || !out)))
        return fail(DGX_ERR_INVALID, "dgx_eval_points: bad argument");
    if (n_points > EVAL_MAX_POINTS)
        return fail(DGX_ERR_INVALID, "dgx_eval_points: at most " + std::to_string(EVAL_MAX_POINTS) + " points");
    std::vector<double> phi((size_t)n_points * c->np), grad(2 * OPS_MAX_NP);
    for (int k = 0; k < n_points; ++k) basis_eval(c->prm.basis, c->prm.order, ref_xy[2 * k], ref_xy[2 * k + 1],
                                                   &phi[(size_t)k * c->np], grad.data());
    if (launch_eval_points(c->ne, c->np, n_points, phi.data(), u, out, (cudaStream_t)stream))
        return fail(DGX_ERR_CUDA, "point evaluation launch failed");
    return DGX_OK;
}

// The host-pointer variants run on the context's own stream and share its scratch buffers
// with calls made on caller streams, so they first wait for all work on the device: a
// synchronous host call is then ordered after every call made before it.
static int ensure_host_buffers(dgx_ctx* c) {
    CUDA_OK(cudaDeviceSynchronize());
    if (c->d_hu) return DGX_OK;
    const size_t sb = (c->nstate ? c->nstate : 1) * sizeof(double);
    if (cudaMalloc((void**)&c->d_hu, sb) != cudaSuccess || cudaMalloc((void**)&c->d_hr, sb) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->host_out, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return fail(DGX_ERR_CUDA, "cudaMalloc failed for host-variant buffers");
    }
    for (cudaEvent_t& e : c->host_ev)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return fail(DGX_ERR_CUDA, "cudaEventCreate failed for host-variant copies");
        }
    return DGX_OK;
}

extern "C" int dgx_residual_host(dgx_ctx* c, const double* u, double* r) {
    if (!c || (c->ne && (!u || !r))) return fail(DGX_ERR_INVALID, "dgx_residual_host: null argument");
    int rc = ensure_host_buffers(c);
    if (rc) return rc;
    const size_t sb = c->nstate * sizeof(double);
    CUDA_OK(cudaMemcpyAsync(c->d_hu, u, sb, cudaMemcpyHostToDevice, c->cap));
    if ((rc = dgx_residual(c, c->d_hu, c->d_hr, c->cap))) return rc;
    CUDA_OK(cudaMemcpyAsync(r, c->d_hr, sb, cudaMemcpyDeviceToHost, c->cap));
    CUDA_OK(cudaStreamSynchronize(c->cap));
    return DGX_OK;
}

// The host-pointer step is bound by the host link (about 210 GB/s in and 193 GB/s out on
// GB300 for pinned memory, copy engines and SM copies alike).  For the CUDA-core mixed forms
// the last step's stage 3, which writes the FP64 state, runs in HOST_CHUNKS tile ranges, and
// each range is copied back on a second stream as soon as it is written, so the copy back
// overlaps the rest of stage 3.
static constexpr int HOST_CHUNKS = 4;

extern "C" int dgx_rk3_step_host(dgx_ctx* c, double* u, double dt, int n_steps) {
    if (!c || (c->ne && !u) || n_steps < 0) return fail(DGX_ERR_INVALID, "dgx_rk3_step_host: bad argument");
    int rc = ensure_host_buffers(c);
    if (rc) return rc;
    const size_t sb = c->nstate * sizeof(double);
    const bool overlap = c->prm.precision == DGX_MIXED && c->nvpe == 3 && c->ne > 0 && n_steps > 0;
    const int ntiles = (c->ne + TILE - 1) / TILE;
    const size_t row = (size_t)c->np * NV;  // doubles per element
    auto tiles_of = [&](int k, int nch, int* t0, int* t1) {
        *t0 = (int)((long long)ntiles * k / nch);
        *t1 = (int)((long long)ntiles * (k + 1) / nch);
    };
    // A single mixed step on a tuned context: the state comes in range by range on the second
    // stream, and each range is converted to FP32 (and its face traces formed) on the context
    // stream while the next range is in flight.
    const bool chunk_in = overlap && n_steps == 1 && c->stage_grid != 0 && ntiles >= HOST_CHUNKS;
    if (!chunk_in) {
        CUDA_OK(cudaMemcpyAsync(c->d_hu, u, sb, cudaMemcpyHostToDevice, c->cap));
    } else {
        for (int k = 0; k < HOST_CHUNKS; ++k) {
            int t0, t1;
            tiles_of(k, HOST_CHUNKS, &t0, &t1);
            const size_t e0 = (size_t)t0 * TILE, e1 = std::min((size_t)t1 * TILE, (size_t)c->ne);
            CUDA_OK(cudaMemcpyAsync(c->d_hu + e0 * row, u + e0 * row, (e1 - e0) * row * sizeof(double),
                                    cudaMemcpyHostToDevice, c->host_out));
            CUDA_OK(cudaEventRecord(c->host_ev[k], c->host_out));
            CUDA_OK(cudaStreamWaitEvent(c->cap, c->host_ev[k], 0));
            if (launch_f64_to_f32((e1 - e0) * row, c->d_hu + e0 * row, c->d_uhi[0] + e0 * row, c->cap))
                return fail(DGX_ERR_CUDA, "conversion launch failed");
            if (c->stage_grid & (STAGE_TRACE | STAGE_TC)) {
                StageArgs t = mixed_stage_args(c, c->d_hu, dt, 0);
                t.tout = c->d_tr[0];
                t.tile0 = t0;
                t.ntile = t1 - t0;
                const int lrc = (c->stage_grid & STAGE_TC)
                                    ? launch_tc_trace_init(c->prm.order, t, c->ops, c->stage_grid & ~STAGE_TC, c->cap)
                                    : launch_trace_init(c->prm.order, t, c->ops, c->cap);
                if (lrc) return fail(DGX_ERR_CUDA, std::string("trace launch failed: ") + launch_error_text());
            }
        }
    }
    if (!overlap) {
        if ((rc = dgx_rk3_step(c, c->d_hu, dt, n_steps, c->cap))) return rc;
        CUDA_OK(cudaMemcpyAsync(u, c->d_hu, sb, cudaMemcpyDeviceToHost, c->cap));
        CUDA_OK(cudaStreamSynchronize(c->cap));
        return DGX_OK;
    }
    // the call's steps but the last, then the last one (STEP_ONLY or STEP_LAST) by hand
    if (n_steps > 1 && (rc = rk3_step_impl(c, c->d_hu, dt, n_steps, c->cap, true))) return rc;
    if (n_steps == 1 && !chunk_in && (rc = mixed_prologue(c, c->d_hu, dt, c->cap))) return rc;
    StageArgs st[3];
    mixed_step_args(c, c->d_hu, dt, (n_steps - 1) & 1, st, n_steps == 1 ? STEP_ONLY : STEP_LAST);
    if ((rc = launch_stage(c, st[0], c->cap)) || (rc = launch_stage(c, st[1], c->cap))) return rc;
    const bool chunked = ntiles >= HOST_CHUNKS;
    const int nch = chunked ? HOST_CHUNKS : 1;
    for (int k = 0; k < nch; ++k) {
        int t0, t1;
        tiles_of(k, nch, &t0, &t1);
        StageArgs a = st[2];
        if (chunked) {
            a.tile0 = t0;
            a.ntile = t1 - t0;
        }
        if ((rc = launch_stage(c, a, c->cap))) return rc;
        CUDA_OK(cudaEventRecord(c->host_ev[k], c->cap));
        CUDA_OK(cudaStreamWaitEvent(c->host_out, c->host_ev[k], 0));
        const size_t e0 = (size_t)t0 * TILE, e1 = std::min((size_t)t1 * TILE, (size_t)c->ne);
        CUDA_OK(cudaMemcpyAsync(u + e0 * row, c->d_hu + e0 * row, (e1 - e0) * row * sizeof(double),
                                cudaMemcpyDeviceToHost, c->host_out));
    }
    CUDA_OK(cudaStreamSynchronize(c->host_out));
    CUDA_OK(cudaStreamSynchronize(c->cap));
    return DGX_OK;
}

extern "C" int dgx_state_alloc(const dgx_ctx* c, double** u) {
    if (!c || !u) return fail(DGX_ERR_INVALID, "dgx_state_alloc: null argument");
    *u = nullptr;
    int dev = -1;
    CUDA_OK(cudaGetDevice(&dev));
    if (dev != c->device) CUDA_OK(cudaSetDevice(c->device));
    const cudaError_t e = cudaMalloc(u, c->nstate ? c->nstate * sizeof(double) : 16);
    if (dev != c->device) cudaSetDevice(dev);
    if (e != cudaSuccess) {
        *u = nullptr;
        return fail(DGX_ERR_CUDA, std::string("dgx_state_alloc: ") + cudaGetErrorString(e));
    }
    return DGX_OK;
}

extern "C" void dgx_state_free(double* u) {
    if (u) cudaFree(u);
}

extern "C" int dgx_state_copy(const dgx_ctx* c, double* dst, const double* src, int to_device) {
    if (!c || (c->nstate && (!dst || !src))) return fail(DGX_ERR_INVALID, "dgx_state_copy: bad argument");
    if (c->nstate == 0) return DGX_OK;
    CUDA_OK(cudaMemcpy(dst, src, c->nstate * sizeof(double), to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost));
    return DGX_OK;
}

extern "C" int dgx_project_host(dgx_ctx* c, const double* uq, double* u) {
    if (!c || (c->ne && (!uq || !u))) return fail(DGX_ERR_INVALID, "dgx_project_host: bad argument");
    if (c->ne == 0) return DGX_OK;
    int rc = ensure_host_buffers(c);
    if (rc) return rc;
    const size_t nq = (size_t)c->ne * c->nq * NV;
    double* d_uq = nullptr;
    CUDA_OK(cudaMalloc(&d_uq, nq * sizeof(double)));
    rc = [&]() -> int {
        CUDA_OK(cudaMemcpyAsync(d_uq, uq, nq * sizeof(double), cudaMemcpyHostToDevice, c->cap));
        if (int r = dgx_project(c, d_uq, c->d_hu, c->cap)) return r;
        CUDA_OK(cudaMemcpyAsync(u, c->d_hu, c->nstate * sizeof(double), cudaMemcpyDeviceToHost, c->cap));
        CUDA_OK(cudaStreamSynchronize(c->cap));
        return DGX_OK;
    }();
    cudaFree(d_uq);
    return rc;
}

extern "C" int dgx_apply_mass_inv_host(dgx_ctx* c, const double* in, double* out) {
    if (!c || (c->ne && (!in || !out))) return fail(DGX_ERR_INVALID, "dgx_apply_mass_inv_host: null argument");
    int rc = ensure_host_buffers(c);
    if (rc) return rc;
    const size_t sb = c->nstate * sizeof(double);
    CUDA_OK(cudaMemcpyAsync(c->d_hu, in, sb, cudaMemcpyHostToDevice, c->cap));
    if ((rc = dgx_apply_mass_inv(c, c->d_hu, c->d_hr, c->cap))) return rc;
    CUDA_OK(cudaMemcpyAsync(out, c->d_hr, sb, cudaMemcpyDeviceToHost, c->cap));
    CUDA_OK(cudaStreamSynchronize(c->cap));
    return DGX_OK;
}

extern "C" int dgx_monitor_host(dgx_ctx* c, const double* u, double dt, double* cfl, double* rho_min,
                                double* rho_max, int* has_nan) {
    if (!c || (c->ne && !u)) return fail(DGX_ERR_INVALID, "dgx_monitor_host: null argument");
    int rc = ensure_host_buffers(c);
    if (rc) return rc;
    CUDA_OK(cudaMemcpyAsync(c->d_hu, u, c->nstate * sizeof(double), cudaMemcpyHostToDevice, c->cap));
    double a = 0.0, lo = 0.0, hi = 0.0;
    int nan = 0;
    if (cfl && (rc = dgx_max_cfl(c, c->d_hu, dt, &a, c->cap))) return rc;
    if ((rho_min || rho_max) && (rc = dgx_density_range(c, c->d_hu, &lo, &hi, c->cap))) return rc;
    if (has_nan && (rc = dgx_has_nan(c, c->d_hu, &nan, c->cap))) return rc;
    CUDA_OK(cudaStreamSynchronize(c->cap));
    if (cfl) *cfl = a;
    if (rho_min) *rho_min = lo;
    if (rho_max) *rho_max = hi;
    if (has_nan) *has_nan = nan;
    return DGX_OK;
}
