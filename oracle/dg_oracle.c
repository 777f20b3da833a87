/*
 * dg_oracle.c -- CPU restatement of dgfem's explicit DG residual-and-update path.
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); see dg_oracle.h.
 *
 * Every function cites the dgfem source it restates (paths inside the dgfem project).
 * The arithmetic follows dgfem's operation order term by term.  The one structural
 * change is that interior-face contributions are first written to per-face buffers
 * and then summed per element in face-list order; that reproduces dgfem's serial
 * accumulation order exactly (assembler.cpp:197-208) while letting the loops run on
 * several threads.
 */
#include "dg_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../discontinuous-galerkin-fem_gb300/csrc/quad_tables.inc"

#define NV 4
#define MAX_TAGS 64

static int g_threads = 1;
void orc_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

/* ------------------------------------------------------------------ quadrature */
/* QuadratureFactory::dunavant_triangle / get_dunavant_rule, factory.cpp:61-73, 238-717 */
int orc_tri_rule(int order, int* n, const double** pts, const double** wts) {
    if (order < 0 || order > DGX_TRI_MAX_ORDER) return -1;
    *n = dgx_tri_rule_npts[order];
    *pts = dgx_tri_rule_points + 2 * dgx_tri_rule_offset[order];
    *wts = dgx_tri_rule_weights + dgx_tri_rule_offset[order];
    return 0;
}

/* QuadratureFactory::gauss_legendre_1d, factory.cpp:16-31, 75-236 */
int orc_gl_rule(int n, const double** pts, const double** wts) {
    if (n < 1 || n > DGX_GL_MAX_POINTS) return -1;
    *pts = dgx_gl_points[n - 1];
    *wts = dgx_gl_weights[n - 1];
    return 0;
}

/* ------------------------------------------------------------------ bases */
int orc_n_basis(int p) { return (p + 1) * (p + 2) / 2; }

/* MonomialBasisTriangle::safe_power, monomial.cpp:24-28 */
static double safe_power(double x, int n) { return n == 0 ? 1.0 : pow(x, (double)n); }

/* MonomialBasisTriangle::evaluate, monomial.cpp:30-43: x^i y^j by total degree, i ascending */
static void monomial_eval(int p, double x, double y, double* phi) {
    int idx = 0;
    for (int td = 0; td <= p; ++td)
        for (int i = 0; i <= td; ++i) {
            int j = td - i;
            phi[idx++] = safe_power(x, i) * safe_power(y, j);
        }
}

/* MonomialBasisTriangle::evaluate_gradient, monomial.cpp:45-72 */
static void monomial_grad(int p, double x, double y, double* g) {
    int idx = 0;
    for (int td = 0; td <= p; ++td)
        for (int i = 0; i <= td; ++i) {
            int j = td - i;
            g[2 * idx] = (i == 0) ? 0.0 : i * safe_power(x, i - 1) * safe_power(y, j);
            g[2 * idx + 1] = (j == 0) ? 0.0 : safe_power(x, i) * j * safe_power(y, j - 1);
            ++idx;
        }
}

/* DubinerBasis::jacobi_polynomial, dubiner.cpp:24-47 */
static double jacobi(int n, double a, double b, double x) {
    if (n == 0) return 1.0;
    if (n == 1) return 0.5 * (a - b + (a + b + 2.0) * x);
    double pm1 = 1.0, pn = 0.5 * (a - b + (a + b + 2.0) * x);
    for (int k = 2; k <= n; ++k) {
        double a1 = 2.0 * k * (k + a + b) * (2.0 * k + a + b - 2.0);
        double a2 = (2.0 * k + a + b - 1.0) * (a * a - b * b);
        double a3 = (2.0 * k + a + b - 2.0) * (2.0 * k + a + b - 1.0) * (2.0 * k + a + b);
        double a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * (2.0 * k + a + b);
        double pp1 = ((a2 + a3 * x) * pn - a4 * pm1) / a1;
        pm1 = pn;
        pn = pp1;
    }
    return pn;
}

/* DubinerBasis::jacobi_derivative, dubiner.cpp:49-53 */
static double jacobi_d(int n, double a, double b, double x) {
    if (n == 0) return 0.0;
    return 0.5 * (n + a + b + 1.0) * jacobi(n - 1, a + 1.0, b + 1.0, x);
}

/* ReferenceTriangle::contains_point / project_to_bounds, elements.cpp:23-25, 58-61 */
static void tri_clamp(double* x, double* y) {
    if (*x >= 0 && *y >= 0 && (*x + *y) <= 1) return;
    *x = fmax(0.0, fmin(1.0, *x));
    *y = fmax(0.0, fmin(1.0 - *x, *y));
}

/* DubinerBasis::get_dubiner_indices, dubiner.cpp:77-90: j outer, i inner */
static void dubiner_ij(int p, int idx, int* oi, int* oj) {
    int k = 0;
    for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p - j; ++i) {
            if (k == idx) { *oi = i; *oj = j; return; }
            ++k;
        }
    *oi = 0; *oj = 0;
}

/* DubinerBasis::evaluate, dubiner.cpp:55-116 */
static void dubiner_eval(int p, double x, double y, double* phi) {
    tri_clamp(&x, &y);
    double ome = 1.0 - y;
    double r = (fabs(ome) < 1e-14) ? -1.0 : 2.0 * x / ome - 1.0;
    double s = 2.0 * y - 1.0;
    int nb = orc_n_basis(p);
    for (int idx = 0; idx < nb; ++idx) {
        int i, j;
        dubiner_ij(p, idx, &i, &j);
        double Pi = jacobi(i, 0.0, 0.0, r);
        double Pj = jacobi(j, 2.0 * i + 1.0, 0.0, s);
        double nrm = 2.0 * sqrt((2.0 * i + 1.0) * (i + j + 1.0));
        double sc = pow(0.5 * (1.0 - s), (double)i);
        phi[idx] = nrm * Pi * Pj * sc;
    }
}

/* DubinerBasis::evaluate_gradient, dubiner.cpp:118-168 */
static void dubiner_grad(int p, double x, double y, double* g) {
    tri_clamp(&x, &y);
    double ome = 1.0 - y;
    double r = (fabs(ome) < 1e-14) ? -1.0 : 2.0 * x / ome - 1.0;
    double s = 2.0 * y - 1.0;
    double dr_dxi, dr_deta, ds_dxi, ds_deta;
    if (fabs(ome) < 1e-14) {
        dr_dxi = dr_deta = ds_dxi = ds_deta = 0.0;
    } else {
        dr_dxi = 2.0 / ome;
        dr_deta = 2.0 * x / (ome * ome);
        ds_dxi = 0.0;
        ds_deta = 2.0;
    }
    int nb = orc_n_basis(p);
    for (int idx = 0; idx < nb; ++idx) {
        int i, j;
        dubiner_ij(p, idx, &i, &j);
        double Pi = jacobi(i, 0.0, 0.0, r);
        double Pj = jacobi(j, 2.0 * i + 1.0, 0.0, s);
        double dPi = (i > 0) ? jacobi_d(i, 0.0, 0.0, r) : 0.0;
        double dPj = (j > 0) ? jacobi_d(j, 2.0 * i + 1.0, 0.0, s) : 0.0;
        double nrm = 2.0 * sqrt((2.0 * i + 1.0) * (i + j + 1.0));
        double sc = pow(0.5 * (1.0 - s), (double)i);
        double dsc = (i > 0) ? -0.5 * i * pow(0.5 * (1.0 - s), (double)(i - 1)) : 0.0;
        double dphi_dr = nrm * dPi * Pj * sc;
        double dphi_ds = nrm * Pi * (dPj * sc + Pj * dsc);
        g[2 * idx] = dphi_dr * dr_dxi + dphi_ds * ds_dxi;
        g[2 * idx + 1] = dphi_dr * dr_deta + dphi_ds * ds_deta;
    }
}

/* LegendreBasis (quads), legendre.cpp:27-110: phi_{i,j} = P_i(x) P_j(y), j outer, i inner;
 * P_n by the three-term recurrence, P'_n by n (x P_n - P_{n-1}) / (x^2 - 1) with the
 * endpoint values n (n+1)/2 (+-1)^(n+1) at |x| = 1 (within 1e-12). */
static void legendre_seq(int p, double x, double* P) {
    P[0] = 1.0;
    if (p >= 1) P[1] = x;
    for (int i = 2; i <= p; ++i) P[i] = ((2 * i - 1) * x * P[i - 1] - (i - 1) * P[i - 2]) / i;
}
static double legendre_d(int n, double x, const double* P) {
    if (n == 0) return 0.0;
    if (fabs(fabs(x) - 1.0) < 1e-12) {
        double sign = x > 0 ? 1.0 : -1.0, parity = (n % 2 == 0) ? 1.0 : -1.0;
        return 0.5 * n * (n + 1) * parity * sign;
    }
    return n * (x * P[n] - P[n - 1]) / (x * x - 1.0);
}
static void legendre_eval(int p, double x, double y, double* phi) {
    double Px[16], Py[16];
    legendre_seq(p, x, Px);
    legendre_seq(p, y, Py);
    int idx = 0;
    for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p; ++i) phi[idx++] = Px[i] * Py[j];
}
static void legendre_grad(int p, double x, double y, double* g) {
    double Px[16], Py[16], dx[16], dy[16];
    legendre_seq(p, x, Px);
    legendre_seq(p, y, Py);
    for (int i = 0; i <= p; ++i) {
        dx[i] = legendre_d(i, x, Px);
        dy[i] = legendre_d(i, y, Py);
    }
    int idx = 0;
    for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p; ++i) {
            g[2 * idx] = dx[i] * Py[j];
            g[2 * idx + 1] = Px[i] * dy[j];
            ++idx;
        }
}

void orc_basis_eval(int basis, int p, double x, double y, double* phi) {
    if (basis == ORC_BASIS_LEGENDRE) legendre_eval(p, x, y, phi);
    else if (basis == ORC_BASIS_DUBINER) dubiner_eval(p, x, y, phi);
    else monomial_eval(p, x, y, phi);
}
void orc_basis_grad(int basis, int p, double x, double y, double* g) {
    if (basis == ORC_BASIS_LEGENDRE) legendre_grad(p, x, y, g);
    else if (basis == ORC_BASIS_DUBINER) dubiner_grad(p, x, y, g);
    else monomial_grad(p, x, y, g);
}

/* ------------------------------------------------------------------ mapping */
/* GeometricMapping::compute_mapping, mapping.cpp:22-50, with the P1 triangle shape
 * functions of ReferenceTriangle::compute_shape_functions, elements.cpp:40-56.
 * J_T = dN^T * vertices; dxi_dx = inverse(J_T) by the 2x2 cofactor formula. */
int orc_compute_mapping_nv(int nv, const double* V, double xi, double eta, double* xp, double* J_det,
                           double* A) {
    double N[4], dN[4][2];
    if (nv == 4) { /* ReferenceQuad::compute_shape_functions, elements.cpp:92-111 */
        N[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
        N[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
        N[2] = 0.25 * (1.0 + xi) * (1.0 + eta);
        N[3] = 0.25 * (1.0 - xi) * (1.0 + eta);
        dN[0][0] = -0.25 * (1.0 - eta); dN[0][1] = -0.25 * (1.0 - xi);
        dN[1][0] = 0.25 * (1.0 - eta);  dN[1][1] = -0.25 * (1.0 + xi);
        dN[2][0] = 0.25 * (1.0 + eta);  dN[2][1] = 0.25 * (1.0 + xi);
        dN[3][0] = -0.25 * (1.0 + eta); dN[3][1] = 0.25 * (1.0 - xi);
    } else {
        N[0] = 1.0 - xi - eta; N[1] = xi; N[2] = eta;
        dN[0][0] = -1.0; dN[0][1] = -1.0; dN[1][0] = 1.0; dN[1][1] = 0.0; dN[2][0] = 0.0; dN[2][1] = 1.0;
    }
    if (xp) {
        xp[0] = xp[1] = 0.0;
        for (int k = 0; k < nv; ++k) {
            xp[0] += N[k] * V[2 * k];
            xp[1] += N[k] * V[2 * k + 1];
        }
    }
    double J[2][2];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) {
            double a = 0.0;
            for (int k = 0; k < nv; ++k) a += dN[k][r] * V[2 * k + c];
            J[r][c] = a;
        }
    double det = J[0][0] * J[1][1] - J[1][0] * J[0][1];
    if (J_det) *J_det = det;
    if (fabs(det) < 1e-12) return -1; /* "Singular Jacobian matrix", mapping.cpp:42-44 */
    if (A) {
        double inv = 1.0 / det;
        A[0] = J[1][1] * inv;
        A[2] = -J[1][0] * inv;
        A[1] = -J[0][1] * inv;
        A[3] = J[0][0] * inv;
    }
    return 0;
}

int orc_compute_mapping(const double* V, double xi, double eta, double* xp, double* J_det, double* A) {
    return orc_compute_mapping_nv(3, V, xi, eta, xp, J_det, A);
}

/* DGSpace::map_face_quad_point, space.cpp:259-288: triangle faces (t, 0), (1-t, t),
 * (0, 1-t) with t = (s+1)/2; quad faces (s, -1), (1, s), (-s, 1), (-1, -s) */
void orc_map_face_point_nv(int nv, int face, double s, double* xi) {
    if (nv == 4) {
        if (face == 0) { xi[0] = s; xi[1] = -1.0; }
        else if (face == 1) { xi[0] = 1.0; xi[1] = s; }
        else if (face == 2) { xi[0] = -s; xi[1] = 1.0; }
        else { xi[0] = -1.0; xi[1] = -s; }
        return;
    }
    double t = 0.5 * (s + 1.0);
    if (face == 0) { xi[0] = t; xi[1] = 0.0; }
    else if (face == 1) { xi[0] = 1.0 - t; xi[1] = t; }
    else { xi[0] = 0.0; xi[1] = 1.0 - t; }
}
void orc_map_face_point(int face, double s, double* xi) { orc_map_face_point_nv(3, face, s, xi); }

/* ReferenceTriangle / ReferenceQuad::edge_vertices, elements.cpp:27-38, 73-90: edge f
 * runs from vertex f to vertex (f + 1) mod nv */
#define EDGE_A(f, nv) (f)
#define EDGE_B(f, nv) (((f) + 1) % (nv))

/* ------------------------------------------------------------------ mesh */
typedef struct {
    int set, type;
    double value[4];
    orc_bc_fn fn;
    void* user;
} orc_bc;

struct orc_mesh {
    int nv, ne;
    int nvpe;  /* vertices (= faces) per element: 3 triangles, 4 quads */
    double* own_q;  /* quads: the tensor Gauss-Legendre rule, [nq][2] points then [nq] weights */
    double* verts;
    int* elems;
    int* nbr;   /* [ne][3][2]  face_neighbors_ */
    int* btag;  /* [ne][3]     boundary_face_tags_ value, -1 when absent */
    /* space */
    int order, basis, np, nq, nfq, space_ready;
    const double *qp, *qw, *fp, *fw;
    double* phi_vol;   /* [nq][np] */
    double* dphi_vol;  /* [nq][np][2] reference gradients */
    double* phi_face;  /* [3][nfq][np] */
    double* jdet;      /* [ne][nq] */
    double* dphi_dx;   /* [ne][nq*np][2] */
    double* fnormal;   /* [ne][3][2] */
    double* flen;      /* [ne][3] */
    double* fqp;       /* [ne][3][2*nfq] column-major flattened */
    double* dphi_dx_face; /* [ne][3][nfq*np][2] */
    /* precomputed faces */
    int nif, nbf;
    int* ifaces;  /* [nif][5] */
    int* bfaces;  /* [nbf][3] */
    int *e2f_off, *e2f;  /* CSR: element -> (face index*2 + side) in face order */
    double *bufL, *bufR, *vbufL, *vbufR;
    double* minv;  /* [ne][np][np] */
    orc_bc bc[MAX_TAGS];
};

typedef struct { int a, b, e, f, ord; } face_rec;

static int face_rec_cmp(const void* x, const void* y) {
    const face_rec* p = (const face_rec*)x;
    const face_rec* q = (const face_rec*)y;
    if (p->a != q->a) return p->a < q->a ? -1 : 1;
    if (p->b != q->b) return p->b < q->b ? -1 : 1;
    return p->ord < q->ord ? -1 : (p->ord > q->ord);
}

/* DGMesh::DGMesh + build_face_connectivity + identify_boundary_faces, mesh.cpp:18-51,
 * 312-402.  Faces keyed by their sorted vertex pair; the first two faces of a key
 * become neighbours (once a key has two entries dgfem connects them and never undoes
 * it).  Boundary tags: a later tag overrides an earlier one for the same edge; faces
 * without a tagged edge get tag 0; with no boundary edges at all no face is tagged. */
orc_mesh* orc_mesh_create_nv(int nvpe, int nv, const double* verts, int ne, const int* elems, int nbe,
                             const int* bedges) {
    if (nvpe != 3 && nvpe != 4) return NULL;
    const int K = nvpe;
    orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
    m->nv = nv;
    m->ne = ne;
    m->nvpe = nvpe;
    m->verts = (double*)malloc(sizeof(double) * 2 * (size_t)(nv ? nv : 1));
    memcpy(m->verts, verts, sizeof(double) * 2 * (size_t)nv);
    m->elems = (int*)malloc(sizeof(int) * K * (size_t)(ne ? ne : 1));
    memcpy(m->elems, elems, sizeof(int) * K * (size_t)ne);
    m->nbr = (int*)malloc(sizeof(int) * 2 * K * (size_t)(ne ? ne : 1));
    for (size_t i = 0; i < 2 * K * (size_t)ne; ++i) m->nbr[i] = -1;
    m->btag = (int*)malloc(sizeof(int) * K * (size_t)(ne ? ne : 1));
    for (size_t i = 0; i < K * (size_t)ne; ++i) m->btag[i] = -1;

    size_t nf = K * (size_t)ne;
    face_rec* r = (face_rec*)malloc(sizeof(face_rec) * (nf ? nf : 1));
    for (int e = 0; e < ne; ++e)
        for (int f = 0; f < K; ++f) {
            int v1 = elems[K * e + f], v2 = elems[K * e + (f + 1) % K];
            face_rec* x = &r[K * e + f];
            x->a = v1 < v2 ? v1 : v2;
            x->b = v1 < v2 ? v2 : v1;
            x->e = e;
            x->f = f;
            x->ord = K * e + f;
        }
    qsort(r, nf, sizeof(face_rec), face_rec_cmp);
    for (size_t i = 0; i < nf;) {
        size_t j = i;
        while (j < nf && r[j].a == r[i].a && r[j].b == r[i].b) ++j;
        if (j - i >= 2) {
            int e1 = r[i].e, f1 = r[i].f, e2 = r[i + 1].e, f2 = r[i + 1].f;
            m->nbr[2 * K * e1 + 2 * f1] = e2;
            m->nbr[2 * K * e1 + 2 * f1 + 1] = f2;
            m->nbr[2 * K * e2 + 2 * f2] = e1;
            m->nbr[2 * K * e2 + 2 * f2 + 1] = f1;
        }
        i = j;
    }
    if (nbe > 0) {
        /* sig -> tag, later entries override: sort boundary edges by (sig, position) */
        face_rec* be = (face_rec*)malloc(sizeof(face_rec) * (size_t)nbe);
        for (int k = 0; k < nbe; ++k) {
            int v1 = bedges[3 * k + 1], v2 = bedges[3 * k + 2];
            be[k].a = v1 < v2 ? v1 : v2;
            be[k].b = v1 < v2 ? v2 : v1;
            be[k].e = bedges[3 * k];
            be[k].ord = k;
        }
        qsort(be, (size_t)nbe, sizeof(face_rec), face_rec_cmp);
        for (int e = 0; e < ne; ++e)
            for (int f = 0; f < K; ++f) {
                if (m->nbr[2 * K * e + 2 * f] != -1) continue;
                int v1 = elems[K * e + f], v2 = elems[K * e + (f + 1) % K];
                face_rec key = {v1 < v2 ? v1 : v2, v1 < v2 ? v2 : v1, 0, 0, 0};
                int lo = 0, hi = nbe, tag = 0;
                while (lo < hi) { /* first entry with sig >= key */
                    int mid = (lo + hi) / 2;
                    if (be[mid].a < key.a || (be[mid].a == key.a && be[mid].b < key.b)) lo = mid + 1;
                    else hi = mid;
                }
                while (lo < nbe && be[lo].a == key.a && be[lo].b == key.b) tag = be[lo++].e;
                m->btag[K * e + f] = tag;
            }
        free(be);
    }
    free(r);
    return m;
}

orc_mesh* orc_mesh_create(int nv, const double* verts, int ne, const int* elems, int nbe, const int* bedges) {
    return orc_mesh_create_nv(3, nv, verts, ne, elems, nbe, bedges);
}

static void mesh_free_space(orc_mesh* m) {
    free(m->phi_vol); free(m->dphi_vol); free(m->phi_face); free(m->jdet); free(m->dphi_dx);
    free(m->fnormal); free(m->flen); free(m->fqp); free(m->dphi_dx_face); free(m->minv); free(m->own_q);
    m->own_q = NULL;
    m->phi_vol = m->dphi_vol = m->phi_face = m->jdet = m->dphi_dx = NULL;
    m->fnormal = m->flen = m->fqp = m->dphi_dx_face = m->minv = NULL;
}

static void mesh_free_faces(orc_mesh* m) {
    free(m->ifaces); free(m->bfaces); free(m->e2f_off); free(m->e2f);
    free(m->bufL); free(m->bufR); free(m->vbufL); free(m->vbufR);
    m->ifaces = m->bfaces = m->e2f_off = m->e2f = NULL;
    m->bufL = m->bufR = m->vbufL = m->vbufR = NULL;
}

void orc_mesh_destroy(orc_mesh* m) {
    if (!m) return;
    mesh_free_space(m);
    mesh_free_faces(m);
    free(m->verts); free(m->elems); free(m->nbr); free(m->btag);
    free(m);
}

static void elem_verts(const orc_mesh* m, int e, double* V) {
    for (int k = 0; k < m->nvpe; ++k) {
        int v = m->elems[m->nvpe * e + k];
        V[2 * k] = m->verts[2 * v];
        V[2 * k + 1] = m->verts[2 * v + 1];
    }
}

/* DGSpace::compute_face_permutation, space.cpp:173-228: true when reversed */
static int face_perm_reversed(int nv, const double* VL, int fL, const double* VR, int fR) {
    const double* a1 = VL + 2 * EDGE_A(fL, nv);
    const double* b1 = VL + 2 * EDGE_B(fL, nv);
    const double* a2 = VR + 2 * EDGE_A(fR, nv);
    const double* b2 = VR + 2 * EDGE_B(fR, nv);
    const double tol = 1e-10;
#define NRM(p, q) sqrt(((p)[0] - (q)[0]) * ((p)[0] - (q)[0]) + ((p)[1] - (q)[1]) * ((p)[1] - (q)[1]))
    int rev = NRM(a1, b2) < tol && NRM(b1, a2) < tol;
    int same = NRM(a1, a2) < tol && NRM(b1, b2) < tol;
#undef NRM
    if (rev || same) return rev;
    double t1[2] = {b1[0] - a1[0], b1[1] - a1[1]};
    double t2[2] = {b2[0] - a2[0], b2[1] - a2[1]};
    double n1 = sqrt(t1[0] * t1[0] + t1[1] * t1[1]);
    double n2 = sqrt(t2[0] * t2[0] + t2[1] * t2[1]);
    t1[0] /= n1; t1[1] /= n1;
    t2[0] /= n2; t2[1] /= n2;
    return (t1[0] * t2[0] + t1[1] * t2[1]) < 0.0;
}

/* open-addressing set of element pairs (build_precomputed_faces' processed set) */
typedef struct { uint64_t* keys; size_t cap; } pair_set;
static int pair_set_insert(pair_set* s, uint64_t k) {
    size_t h = (size_t)((k * 0x9E3779B97F4A7C15ull) >> 17) & (s->cap - 1);
    while (s->keys[h] != UINT64_MAX) {
        if (s->keys[h] == k) return 0;
        h = (h + 1) & (s->cap - 1);
    }
    s->keys[h] = k;
    return 1;
}

/* DGMesh::build_precomputed_faces, mesh.cpp:404-480: interior faces de-duplicated by
 * element pair, in element-then-face order; everything else is a boundary face. */
int orc_mesh_rebuild_faces(orc_mesh* m) {
    mesh_free_faces(m);
    int ne = m->ne;
    const int K = m->nvpe;
    m->ifaces = (int*)malloc(sizeof(int) * 5 * (size_t)(ne ? ne : 1) * K);
    m->bfaces = (int*)malloc(sizeof(int) * 3 * (size_t)(ne ? ne : 1) * K);
    pair_set ps;
    ps.cap = 1;
    while (ps.cap < (size_t)ne * 4 + 16) ps.cap <<= 1;
    ps.keys = (uint64_t*)malloc(sizeof(uint64_t) * ps.cap);
    memset(ps.keys, 0xff, sizeof(uint64_t) * ps.cap);
    int nif = 0, nbf = 0;
    double VL[8], VR[8];
    for (int L = 0; L < ne; ++L) {
        elem_verts(m, L, VL);
        for (int fL = 0; fL < K; ++fL) {
            int R = m->nbr[2 * K * L + 2 * fL], fR = m->nbr[2 * K * L + 2 * fL + 1];
            if (R >= 0) {
                uint64_t lo = (uint64_t)(L < R ? L : R), hi = (uint64_t)(L < R ? R : L);
                if (pair_set_insert(&ps, (lo << 32) | hi)) {
                    elem_verts(m, R, VR);
                    int* F = &m->ifaces[5 * nif++];
                    F[0] = L; F[1] = R; F[2] = fL; F[3] = fR;
                    F[4] = face_perm_reversed(K, VL, fL, VR, fR);
                }
            } else {
                int* B = &m->bfaces[3 * nbf++];
                B[0] = L; B[1] = fL; B[2] = m->btag[K * L + fL];
            }
        }
    }
    free(ps.keys);
    m->nif = nif;
    m->nbf = nbf;
    /* element -> interior faces in face order */
    m->e2f_off = (int*)calloc((size_t)ne + 1, sizeof(int));
    m->e2f = (int*)malloc(sizeof(int) * 2 * (size_t)(nif > 0 ? nif : 1));
    for (int k = 0; k < nif; ++k) {
        m->e2f_off[m->ifaces[5 * k] + 1]++;
        m->e2f_off[m->ifaces[5 * k + 1] + 1]++;
    }
    for (int e = 0; e < ne; ++e) m->e2f_off[e + 1] += m->e2f_off[e];
    int* fill = (int*)calloc((size_t)ne, sizeof(int));
    for (int k = 0; k < nif; ++k) {
        int L = m->ifaces[5 * k], R = m->ifaces[5 * k + 1];
        m->e2f[m->e2f_off[L] + fill[L]++] = 2 * k;
        m->e2f[m->e2f_off[R] + fill[R]++] = 2 * k + 1;
    }
    free(fill);
    return 0;
}

/* DGMesh::set_periodic_boundaries, mesh.cpp:482-588 */
int orc_mesh_set_periodic(orc_mesh* m, int tag1, int tag2, int match_on_y) {
    int ne = m->ne;
    const int K = m->nvpe;
    int *f1 = (int*)malloc(sizeof(int) * K * (size_t)(ne ? ne : 1)), *f2 = (int*)malloc(sizeof(int) * K * (size_t)(ne ? ne : 1));
    int n1 = 0, n2 = 0;
    for (int i = 0; i < K * ne; ++i) { /* boundary_face_tags_ iterates in (elem, face) order */
        if (m->btag[i] < 0) continue;
        if (m->btag[i] == tag1) f1[n1++] = i;
        else if (m->btag[i] == tag2) f2[n2++] = i;
    }
    if (n1 == 0 || n2 == 0) { free(f1); free(f2); return -1; }
    double* c2 = (double*)malloc(sizeof(double) * (size_t)n2);
    for (int k = 0; k < n2; ++k) {
        int e = f2[k] / K, f = f2[k] % K;
        int va = m->elems[K * e + f], vb = m->elems[K * e + (f + 1) % K];
        int c = match_on_y ? 1 : 0;
        c2[k] = 0.5 * (m->verts[2 * va + c] + m->verts[2 * vb + c]);
    }
    for (int k = 0; k < n1; ++k) {
        int e1 = f1[k] / K, l1 = f1[k] % K;
        int va = m->elems[K * e1 + l1], vb = m->elems[K * e1 + (l1 + 1) % K];
        int c = match_on_y ? 1 : 0;
        double c1 = 0.5 * (m->verts[2 * va + c] + m->verts[2 * vb + c]);
        double best = 1.79769313486231570815e308;
        int bi = -1;
        for (int j = 0; j < n2; ++j) {
            double d = fabs(c1 - c2[j]);
            if (d < best) { best = d; bi = j; }
        }
        if (bi >= 0) {
            int e2 = f2[bi] / K, l2 = f2[bi] % K;
            m->nbr[2 * K * e1 + 2 * l1] = e2;
            m->nbr[2 * K * e1 + 2 * l1 + 1] = l2;
            m->nbr[2 * K * e2 + 2 * l2] = e1;
            m->nbr[2 * K * e2 + 2 * l2 + 1] = l1;
        }
    }
    free(c2); free(f1); free(f2);
    if (m->space_ready) orc_mesh_rebuild_faces(m);
    return 0;
}

/* DGSpace ctor + precompute_basis_values + DGMesh::initialize_dg_space,
 * space.cpp:20-67, 69-171, 230-257; mesh.cpp:53-99 */
int orc_mesh_init_space(orc_mesh* m, int order, int basis) {
    if (order < 1 || order > 10) return -1;
    const int K = m->nvpe;
    if (K == 4 && basis != ORC_BASIS_LEGENDRE) return -1; /* DGSpace::create_basis, space.cpp:307-319 */
    if (K == 3 && basis == ORC_BASIS_LEGENDRE) return -1;
    int nq;
    mesh_free_space(m);
    if (K == 3) {
        if (orc_tri_rule(2 * order, &nq, &m->qp, &m->qw)) return -1;
    } else { /* QuadratureFactory::gauss_legendre_quad, factory.cpp:33-59: j outer, i inner */
        const double *gp, *gw;
        if (orc_gl_rule(order + 1, &gp, &gw)) return -1;
        int n1 = order + 1;
        nq = n1 * n1;
        m->own_q = (double*)malloc(sizeof(double) * 3 * nq);
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n1; ++i) {
                int q = j * n1 + i;
                m->own_q[2 * q] = gp[i];
                m->own_q[2 * q + 1] = gp[j];
                m->own_q[2 * nq + q] = gw[i] * gw[j];
            }
        m->qp = m->own_q;
        m->qw = m->own_q + 2 * nq;
    }
    if (orc_gl_rule(order + 1, &m->fp, &m->fw)) return -1;
    m->order = order;
    m->basis = basis;
    int np = m->np = K == 3 ? orc_n_basis(order) : (order + 1) * (order + 1);
    m->nq = nq;
    int nfq = m->nfq = order + 1;
    int ne = m->ne;
    m->phi_vol = (double*)malloc(sizeof(double) * nq * np);
    m->dphi_vol = (double*)malloc(sizeof(double) * nq * np * 2);
    m->phi_face = (double*)malloc(sizeof(double) * K * nfq * np);
    for (int q = 0; q < nq; ++q) {
        orc_basis_eval(basis, order, m->qp[2 * q], m->qp[2 * q + 1], m->phi_vol + q * np);
        orc_basis_grad(basis, order, m->qp[2 * q], m->qp[2 * q + 1], m->dphi_vol + q * np * 2);
    }
    for (int f = 0; f < K; ++f)
        for (int q = 0; q < nfq; ++q) {
            double xi[2];
            orc_map_face_point_nv(K, f, m->fp[q], xi);
            orc_basis_eval(basis, order, xi[0], xi[1], m->phi_face + (f * nfq + q) * np);
        }
    size_t nes = ne ? (size_t)ne : 1;
    m->jdet = (double*)malloc(sizeof(double) * nes * nq);
    m->dphi_dx = (double*)malloc(sizeof(double) * nes * nq * np * 2);
    m->fnormal = (double*)malloc(sizeof(double) * nes * 2 * K);
    m->flen = (double*)malloc(sizeof(double) * nes * K);
    m->fqp = (double*)malloc(sizeof(double) * nes * K * 2 * nfq);
    m->dphi_dx_face = (double*)malloc(sizeof(double) * nes * K * nfq * np * 2);
    double* gface = (double*)malloc(sizeof(double) * K * nfq * np * 2);
    for (int f = 0; f < K; ++f)
        for (int q = 0; q < nfq; ++q) {
            double xi[2];
            orc_map_face_point_nv(K, f, m->fp[q], xi);
            orc_basis_grad(basis, order, xi[0], xi[1], gface + (f * nfq + q) * np * 2);
        }
    int err = 0;
    for (int e = 0; e < ne; ++e) {
        double V[8], A[4], det;
        elem_verts(m, e, V);
        /* compute_element_data, space.cpp:69-102 */
        for (int q = 0; q < nq; ++q) {
            if (orc_compute_mapping_nv(K, V, m->qp[2 * q], m->qp[2 * q + 1], NULL, &det, A)) err = -2;
            m->jdet[(size_t)e * nq + q] = det;
            for (int i = 0; i < np; ++i) {
                const double* g = m->dphi_vol + (q * np + i) * 2;
                double* o = m->dphi_dx + ((size_t)e * nq * np + q * np + i) * 2;
                o[0] = A[0] * g[0] + A[1] * g[1];
                o[1] = A[2] * g[0] + A[3] * g[1];
            }
        }
        /* compute_face_data, space.cpp:104-171 */
        double cx = 0.0, cy = 0.0;
        for (int k = 0; k < K; ++k) {
            cx += V[2 * k];
            cy += V[2 * k + 1];
        }
        cx /= K;
        cy /= K;
        for (int f = 0; f < K; ++f) {
            const double* v1 = V + 2 * EDGE_A(f, K);
            const double* v2 = V + 2 * EDGE_B(f, K);
            double tx = v2[0] - v1[0], ty = v2[1] - v1[1];
            double len = sqrt(tx * tx + ty * ty);
            if (len < 1e-14) err = -3; /* "Degenerate edge detected" */
            double nx = ty / len, ny = -tx / len;
            double mx = 0.5 * (v1[0] + v2[0]), my = 0.5 * (v1[1] + v2[1]);
            if (nx * (mx - cx) + ny * (my - cy) < 0) { nx = -nx; ny = -ny; }
            m->fnormal[(size_t)e * 2 * K + 2 * f] = nx;
            m->fnormal[(size_t)e * 2 * K + 2 * f + 1] = ny;
            m->flen[(size_t)e * K + f] = len;
            double* qpo = m->fqp + ((size_t)e * K + f) * 2 * nfq;
            for (int q = 0; q < nfq; ++q) {
                double t = 0.5 * (m->fp[q] + 1.0);
                qpo[q] = (1.0 - t) * v1[0] + t * v2[0];
                qpo[q + nfq] = (1.0 - t) * v1[1] + t * v2[1];
                double xi[2];
                orc_map_face_point_nv(K, f, m->fp[q], xi);
                if (orc_compute_mapping_nv(K, V, xi[0], xi[1], NULL, &det, A)) err = -2;
                for (int i = 0; i < np; ++i) {
                    const double* g = gface + ((f * nfq + q) * np + i) * 2;
                    double* o = m->dphi_dx_face + (((size_t)e * K + f) * nfq * np + q * np + i) * 2;
                    o[0] = A[0] * g[0] + A[1] * g[1];
                    o[1] = A[2] * g[0] + A[3] * g[1];
                }
            }
        }
    }
    free(gface);
    if (err) return err;
    m->space_ready = 1;
    return orc_mesh_rebuild_faces(m);
}

int orc_mesh_n_interior_faces(const orc_mesh* m) { return m->nif; }
int orc_mesh_n_boundary_faces(const orc_mesh* m) { return m->nbf; }
void orc_mesh_interior_faces(const orc_mesh* m, int* out) {
    memcpy(out, m->ifaces, sizeof(int) * 5 * (size_t)m->nif);
}
void orc_mesh_boundary_faces(const orc_mesh* m, int* out) {
    memcpy(out, m->bfaces, sizeof(int) * 3 * (size_t)m->nbf);
}
void orc_mesh_neighbors(const orc_mesh* m, int* out) {
    memcpy(out, m->nbr, sizeof(int) * 2 * m->nvpe * (size_t)m->ne);
}
int orc_mesh_nvpe(const orc_mesh* m) { return m->nvpe; }
void orc_mesh_space_dims(const orc_mesh* m, int* np, int* nq, int* nfq) {
    *np = m->np; *nq = m->nq; *nfq = m->nfq;
}
void orc_mesh_element_data(const orc_mesh* m, int e, double* J_det, double* dphi_dx) {
    memcpy(J_det, m->jdet + (size_t)e * m->nq, sizeof(double) * m->nq);
    memcpy(dphi_dx, m->dphi_dx + (size_t)e * m->nq * m->np * 2, sizeof(double) * m->nq * m->np * 2);
}
void orc_mesh_face_data(const orc_mesh* m, int e, int f, double* normal, double* length,
                        double* quad_points, double* dphi_dx_face) {
    const int K = m->nvpe;
    normal[0] = m->fnormal[(size_t)e * 2 * K + 2 * f];
    normal[1] = m->fnormal[(size_t)e * 2 * K + 2 * f + 1];
    *length = m->flen[(size_t)e * K + f];
    memcpy(quad_points, m->fqp + ((size_t)e * K + f) * 2 * m->nfq, sizeof(double) * 2 * m->nfq);
    memcpy(dphi_dx_face, m->dphi_dx_face + ((size_t)e * K + f) * m->nfq * m->np * 2,
           sizeof(double) * m->nfq * m->np * 2);
}
void orc_space_tables(const orc_mesh* m, double* phi_vol, double* phi_face, double* vol_w,
                      double* face_w) {
    memcpy(phi_vol, m->phi_vol, sizeof(double) * m->nq * m->np);
    memcpy(phi_face, m->phi_face, sizeof(double) * m->nvpe * m->nfq * m->np);
    memcpy(vol_w, m->qw, sizeof(double) * m->nq);
    memcpy(face_w, m->fw, sizeof(double) * m->nfq);
}

/* GeometricMapping::map_to_physical (mapping.cpp:52-58) at every volume point */
void orc_mesh_quad_points(const orc_mesh* m, double* xq) {
    for (int e = 0; e < m->ne; ++e) {
        double V[8];
        elem_verts(m, e, V);
        for (int q = 0; q < m->nq; ++q)
            orc_compute_mapping_nv(m->nvpe, V, m->qp[2 * q], m->qp[2 * q + 1], xq + ((size_t)e * m->nq + q) * 2,
                                   NULL, NULL);
    }
}

int orc_mesh_set_bc(orc_mesh* m, int tag, int type, const double* value4, orc_bc_fn fn,
                    void* user) {
    if (tag < 0 || tag >= MAX_TAGS) return -1;
    orc_bc* b = &m->bc[tag];
    b->set = 1;
    b->type = type;
    for (int v = 0; v < 4; ++v) b->value[v] = value4 ? value4[v] : 0.0;
    b->fn = fn;
    b->user = user;
    return 0;
}

/* BoundaryConditionEuler::evaluate, conditions.cpp:54-60 */
static void bc_eval(const orc_bc* b, double x, double y, double* out) {
    if (b->fn) b->fn(x, y, out, b->user);
    else for (int v = 0; v < 4; ++v) out[v] = b->value[v];
}

/* ------------------------------------------------------------------ physics */
/* conserved_to_primitive, euler_weak_formulation.cpp:279-296 */
static void c2p(const double* U, double gamma, double* W) {
    double rho = U[0];
    double rho_inv = 1.0 / rho;
    double u = U[1] * rho_inv, v = U[2] * rho_inv;
    double gm1 = gamma - 1.0;
    W[0] = rho; W[1] = u; W[2] = v;
    W[3] = gm1 * (U[3] - 0.5 * rho * (u * u + v * v));
}

/* primitive_to_conserved, euler_weak_formulation.cpp:261-277 */
static void p2c(const double* W, double gamma, double* U) {
    double rho = W[0], u = W[1], v = W[2], p = W[3];
    double gm1 = gamma - 1.0;
    U[0] = rho; U[1] = rho * u; U[2] = rho * v;
    U[3] = p / gm1 + 0.5 * rho * (u * u + v * v);
}

/* get_fluxes_and_primitive, euler_weak_formulation.cpp:27-43 */
static void fluxes(const double* U, double gamma, double* F, double* G, double* W) {
    c2p(U, gamma, W);
    double rho = W[0], u = W[1], v = W[2], p = W[3];
    double E = U[3];
    F[0] = U[1]; F[1] = rho * u * u + p; F[2] = rho * u * v; F[3] = u * (E + p);
    G[0] = U[2]; G[1] = rho * u * v; G[2] = rho * v * v + p; G[3] = v * (E + p);
}

/* EulerWeakFormulation::rusanov_flux, euler_weak_formulation.cpp:51-70 */
void orc_rusanov(double gamma, const double* UL, const double* UR, const double* n, double* H) {
    double FL[4], GL[4], WL[4], FR[4], GR[4], WR[4];
    fluxes(UL, gamma, FL, GL, WL);
    fluxes(UR, gamma, FR, GR, WR);
    double cL = sqrt(gamma * WL[3] / WL[0]);
    double cR = sqrt(gamma * WR[3] / WR[0]);
    double unL = WL[1] * n[0] + WL[2] * n[1];
    double unR = WR[1] * n[0] + WR[2] * n[1];
    double a = fabs(unL) + cL, b = fabs(unR) + cR;
    double smax = (a < b) ? b : a;
    double hs = 0.5 * smax;
    for (int v = 0; v < 4; ++v) {
        double FnL = FL[v] * n[0] + GL[v] * n[1];
        double FnR = FR[v] * n[0] + GR[v] * n[1];
        H[v] = 0.5 * (FnL + FnR) - hs * (UR[v] - UL[v]);
    }
}

/* NavierStokesWeakFormulation::compute_primitive_gradients + compute_viscous_fluxes,
 * navier_stokes_weak_formulation.cpp:36-98 (gas constant 1) */
void orc_viscous_flux(const orc_physics* ph, const double* U, const double* gU, double* Fv,
                      double* Gv) {
    const double gamma = ph->gamma, mu = ph->mu, R = 1.0;
    double rho_safe = fmax(U[0], 1e-12);
    double W[4];
    c2p(U, gamma, W);
    double rho = W[0], u = W[1], v = W[2], p = W[3];
    double grho[2] = {gU[0], gU[1]}, grhou[2] = {gU[2], gU[3]};
    double grhov[2] = {gU[4], gU[5]}, gE[2] = {gU[6], gU[7]};
    double rho_inv = 1.0 / rho_safe;
    double gu[2], gv[2], gp[2], gT[2];
    for (int c = 0; c < 2; ++c) {
        gu[c] = (grhou[c] - u * grho[c]) * rho_inv;
        gv[c] = (grhov[c] - v * grho[c]) * rho_inv;
    }
    double ksq = u * u + v * v;
    for (int c = 0; c < 2; ++c) {
        double mom = rho * (u * gu[c] + v * gv[c]);
        gp[c] = (gamma - 1.0) * (gE[c] - 0.5 * ksq * grho[c] - mom);
    }
    double rho_sq = rho * rho;
    for (int c = 0; c < 2; ++c) gT[c] = (rho * gp[c] - p * grho[c]) / (rho_sq * R);
    double div = gu[0] + gv[1];
    double lambda = -2.0 * mu / 3.0;
    double txx = 2.0 * mu * gu[0] + lambda * div;
    double tyy = 2.0 * mu * gv[1] + lambda * div;
    double txy = mu * (gu[1] + gv[0]);
    double kappa = mu * gamma / (ph->prandtl * (gamma - 1.0));
    double qx = -kappa * gT[0], qy = -kappa * gT[1];
    Fv[0] = 0.0; Fv[1] = txx; Fv[2] = txy; Fv[3] = u * txx + v * txy + qx;
    Gv[0] = 0.0; Gv[1] = txy; Gv[2] = tyy; Gv[3] = u * txy + v * tyy + qy;
}

/* NavierStokesWeakFormulation::compute_penalty_parameter, :275-278 */
double orc_penalty(const orc_physics* ph, int p, double h) {
    double hs = fmax(h, 1e-12);
    return ph->sigma0 * ph->mu * (double)(p + 1) * (double)(p + 1) / hs;
}

#define UE(u, e, np) ((u) + (size_t)(e) * (np) * NV)

/* EulerWeakFormulation::volume_residual, euler_weak_formulation.cpp:72-115 */
int orc_volume_residual(const orc_mesh* m, const orc_physics* ph, int e, const double* u,
                        double* R) {
    int np = m->np, nq = m->nq;
    const double* ue = UE(u, e, np);
    const double* J = m->jdet + (size_t)e * nq;
    const double* D = m->dphi_dx + (size_t)e * nq * np * 2;
    memset(R, 0, sizeof(double) * np * NV);
    for (int q = 0; q < nq; ++q) {
        double U[4] = {0, 0, 0, 0};
        for (int i = 0; i < np; ++i)
            for (int v = 0; v < NV; ++v) U[v] += m->phi_vol[q * np + i] * ue[i * NV + v];
        double F[4], G[4], W[4];
        fluxes(U, ph->gamma, F, G, W);
        double w = m->qw[q] * fabs(J[q]);
        for (int i = 0; i < np; ++i) {
            double dx = D[(q * np + i) * 2], dy = D[(q * np + i) * 2 + 1];
            for (int v = 0; v < NV; ++v) R[i * NV + v] += w * (dx * F[v] + dy * G[v]);
        }
    }
    return 0;
}

/* NavierStokesWeakFormulation::viscous_volume_residual, :100-140 */
int orc_viscous_volume_residual(const orc_mesh* m, const orc_physics* ph, int e, const double* u,
                                double* R) {
    int np = m->np, nq = m->nq;
    const double* ue = UE(u, e, np);
    const double* J = m->jdet + (size_t)e * nq;
    const double* D = m->dphi_dx + (size_t)e * nq * np * 2;
    memset(R, 0, sizeof(double) * np * NV);
    for (int q = 0; q < nq; ++q) {
        double U[4] = {0, 0, 0, 0}, gU[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < np; ++i)
            for (int v = 0; v < NV; ++v) U[v] += m->phi_vol[q * np + i] * ue[i * NV + v];
        for (int i = 0; i < np; ++i) {
            double gx = D[(q * np + i) * 2], gy = D[(q * np + i) * 2 + 1];
            for (int v = 0; v < NV; ++v) {
                gU[2 * v] += ue[i * NV + v] * gx;
                gU[2 * v + 1] += ue[i * NV + v] * gy;
            }
        }
        double Fv[4], Gv[4];
        orc_viscous_flux(ph, U, gU, Fv, Gv);
        double w = m->qw[q] * fabs(J[q]);
        for (int i = 0; i < np; ++i) {
            double gx = D[(q * np + i) * 2], gy = D[(q * np + i) * 2 + 1];
            for (int v = 0; v < NV; ++v) R[i * NV + v] -= w * (Fv[v] * gx + Gv[v] * gy);
        }
    }
    return 0;
}

/* EulerWeakFormulation::interior_face_residual (euler_weak_formulation.cpp:117-175) and
 * NavierStokesWeakFormulation::viscous_interior_face_residual (:142-207) */
int orc_interior_face_residual(const orc_mesh* m, const orc_physics* ph, int k, const double* u,
                               int viscous, double* RL, double* RR) {
    int np = m->np, nfq = m->nfq;
    const int* F = m->ifaces + 5 * k;
    int L = F[0], Rr = F[1], fL = F[2], fR = F[3], rev = F[4];
    const double* uL = UE(u, L, np);
    const double* uR = UE(u, Rr, np);
    const double* phiL = m->phi_face + fL * nfq * np;
    const double* phiR = m->phi_face + fR * nfq * np;
    const int K = m->nvpe;
    const double* n = m->fnormal + (size_t)L * 2 * K + 2 * fL;
    double hF = m->flen[(size_t)L * K + fL];
    const double* gL = m->dphi_dx_face + ((size_t)L * K + fL) * nfq * np * 2;
    const double* gR = m->dphi_dx_face + ((size_t)Rr * K + fR) * nfq * np * 2;
    double sigma = viscous ? orc_penalty(ph, m->order, hF) : 0.0;
    memset(RL, 0, sizeof(double) * np * NV);
    memset(RR, 0, sizeof(double) * np * NV);
    for (int q = 0; q < nfq; ++q) {
        int qR = rev ? nfq - 1 - q : q;
        double ULq[4] = {0, 0, 0, 0}, URq[4] = {0, 0, 0, 0}, Fn[4];
        for (int i = 0; i < np; ++i) {
            double pL = phiL[q * np + i], pR = phiR[qR * np + i];
            for (int v = 0; v < NV; ++v) {
                ULq[v] += pL * uL[i * NV + v];
                URq[v] += pR * uR[i * NV + v];
            }
        }
        if (!viscous) {
            orc_rusanov(ph->gamma, ULq, URq, n, Fn);
        } else {
            double gUL[8] = {0}, gUR[8] = {0};
            for (int i = 0; i < np; ++i) {
                const double* a = gL + (q * np + i) * 2;
                const double* b = gR + (qR * np + i) * 2;
                for (int v = 0; v < NV; ++v) {
                    gUL[2 * v] += uL[i * NV + v] * a[0];
                    gUL[2 * v + 1] += uL[i * NV + v] * a[1];
                    gUR[2 * v] += uR[i * NV + v] * b[0];
                    gUR[2 * v + 1] += uR[i * NV + v] * b[1];
                }
            }
            double FvL[4], GvL[4], FvR[4], GvR[4];
            orc_viscous_flux(ph, ULq, gUL, FvL, GvL);
            orc_viscous_flux(ph, URq, gUR, FvR, GvR);
            for (int v = 0; v < NV; ++v) {
                double avg = 0.5 * (FvL[v] * n[0] + GvL[v] * n[1]);
                avg += 0.5 * (FvR[v] * (-n[0]) + GvR[v] * (-n[1]));
                Fn[v] = avg - sigma * (URq[v] - ULq[v]);
            }
        }
        double w = m->fw[q] * hF * 0.5;
        for (int i = 0; i < np; ++i) {
            double sL = w * phiL[q * np + i], sR = w * phiR[qR * np + i];
            for (int v = 0; v < NV; ++v) {
                RL[i * NV + v] -= sL * Fn[v];
                RR[i * NV + v] += sR * Fn[v];
            }
        }
    }
    return 0;
}

/* EulerWeakFormulation::boundary_face_residual (euler_weak_formulation.cpp:177-250) and
 * NavierStokesWeakFormulation::viscous_boundary_face_residual (:209-273).  The Euler
 * version reads the face points through a row-major view of column-major data
 * (:190-194, 210); the viscous version reads them correctly (:243-247). */
int orc_boundary_face_residual(const orc_mesh* m, const orc_physics* ph, int k, const double* u,
                               int viscous, double* R) {
    int np = m->np, nfq = m->nfq;
    int e = m->bfaces[3 * k], f = m->bfaces[3 * k + 1], tag = m->bfaces[3 * k + 2];
    const orc_bc* bc = (tag >= 0 && tag < MAX_TAGS && m->bc[tag].set) ? &m->bc[tag] : NULL;
    const double* ue = UE(u, e, np);
    const double* phi = m->phi_face + f * nfq * np;
    const int K = m->nvpe;
    const double* n = m->fnormal + (size_t)e * 2 * K + 2 * f;
    double hF = m->flen[(size_t)e * K + f];
    const double* qp = m->fqp + ((size_t)e * K + f) * 2 * nfq;
    const double* g = m->dphi_dx_face + ((size_t)e * K + f) * nfq * np * 2;
    double sigma = viscous ? orc_penalty(ph, m->order, hF) : 0.0;
    memset(R, 0, sizeof(double) * np * NV);
    if (!viscous && !bc) return -1;
    for (int q = 0; q < nfq; ++q) {
        double UL[4] = {0, 0, 0, 0}, Fn[4];
        for (int i = 0; i < np; ++i)
            for (int v = 0; v < NV; ++v) UL[v] += phi[q * np + i] * ue[i * NV + v];
        if (!viscous) {
            double WL[4], UR[4];
            c2p(UL, ph->gamma, WL);
            double xq = qp[2 * q], yq = qp[2 * q + 1]; /* row-major view, :193-194, 210 */
            if (bc->type == ORC_BC_FAR_FIELD) {
                bc_eval(bc, xq, yq, UR);
            } else if (bc->type == ORC_BC_SLIP_WALL) {
                double un = WL[1] * n[0] + WL[2] * n[1];
                double unx = un * n[0], uny = un * n[1];
                double utx = WL[1] - unx, uty = WL[2] - uny;
                double WR[4] = {WL[0], utx - unx, uty - uny, WL[3]};
                p2c(WR, ph->gamma, UR);
            } else if (bc->type == ORC_BC_NO_SLIP_WALL) {
                double Wb[4];
                bc_eval(bc, xq, yq, Wb);
                p2c(Wb, ph->gamma, UR);
            } else {
                return -2; /* PERIODIC boundary face: dgfem throws */
            }
            orc_rusanov(ph->gamma, UL, UR, n, Fn);
        } else {
            double gU[8] = {0};
            for (int i = 0; i < np; ++i) {
                const double* a = g + (q * np + i) * 2;
                for (int v = 0; v < NV; ++v) {
                    gU[2 * v] += ue[i * NV + v] * a[0];
                    gU[2 * v + 1] += ue[i * NV + v] * a[1];
                }
            }
            double Fv[4], Gv[4], Ub[4] = {UL[0], UL[1], UL[2], UL[3]};
            orc_viscous_flux(ph, UL, gU, Fv, Gv);
            if (bc) {
                double data[4];
                bc_eval(bc, qp[q], qp[q + nfq], data);
                if (bc->type == ORC_BC_NO_SLIP_WALL) p2c(data, ph->gamma, Ub);
                else for (int v = 0; v < 4; ++v) Ub[v] = data[v];
            }
            for (int v = 0; v < NV; ++v)
                Fn[v] = (Fv[v] * n[0] + Gv[v] * n[1]) - sigma * (Ub[v] - UL[v]);
        }
        double w = m->fw[q] * hF * 0.5;
        for (int i = 0; i < np; ++i) {
            double s = w * phi[q * np + i];
            for (int v = 0; v < NV; ++v) R[i * NV + v] -= s * Fn[v];
        }
    }
    return 0;
}

/* DGAssembler::assemble_euler_residual, assembler.cpp:137-279: volume, viscous volume,
 * interior faces, viscous interior faces, boundary faces, viscous boundary faces. */
int orc_assemble_residual(const orc_mesh* m, const orc_physics* ph, const double* u, double* R) {
    orc_mesh* mm = (orc_mesh*)m;
    int np = m->np, ne = m->ne, nif = m->nif;
    size_t blk = (size_t)np * NV;
    int visc = ph->viscous;
    if (!m->space_ready) return -1;
    if (!mm->bufL && nif > 0) {
        mm->bufL = (double*)malloc(sizeof(double) * blk * nif);
        mm->bufR = (double*)malloc(sizeof(double) * blk * nif);
    }
    if (visc && !mm->vbufL && nif > 0) {
        mm->vbufL = (double*)malloc(sizeof(double) * blk * nif);
        mm->vbufR = (double*)malloc(sizeof(double) * blk * nif);
    }
    int err = 0;
#pragma omp parallel num_threads(g_threads) reduction(| : err)
    {
        double tmp[64 * NV];
#pragma omp for schedule(static)
        for (int e = 0; e < ne; ++e) {
            err |= orc_volume_residual(m, ph, e, u, R + e * blk);
            if (visc) {
                err |= orc_viscous_volume_residual(m, ph, e, u, tmp);
                for (size_t j = 0; j < blk; ++j) R[e * blk + j] += tmp[j];
            }
        }
#pragma omp for schedule(static)
        for (int k = 0; k < nif; ++k) {
            err |= orc_interior_face_residual(m, ph, k, u, 0, mm->bufL + k * blk, mm->bufR + k * blk);
            if (visc)
                err |= orc_interior_face_residual(m, ph, k, u, 1, mm->vbufL + k * blk,
                                                  mm->vbufR + k * blk);
        }
#pragma omp for schedule(static)
        for (int e = 0; e < ne; ++e) {
            for (int pass = 0; pass < (visc ? 2 : 1); ++pass) {
                const double* bL = pass ? mm->vbufL : mm->bufL;
                const double* bR = pass ? mm->vbufR : mm->bufR;
                for (int t = m->e2f_off[e]; t < m->e2f_off[e + 1]; ++t) {
                    int k = m->e2f[t] >> 1, side = m->e2f[t] & 1;
                    const double* src = (side ? bR : bL) + (size_t)k * blk;
                    for (size_t j = 0; j < blk; ++j) R[e * blk + j] += src[j];
                }
            }
        }
    }
    double tmp[64 * NV];
    for (int k = 0; k < m->nbf; ++k) {
        int tag = m->bfaces[3 * k + 2];
        if (tag < 0 || tag >= MAX_TAGS || !m->bc[tag].set) continue;
        if (orc_boundary_face_residual(m, ph, k, u, 0, tmp)) return -2;
        int e = m->bfaces[3 * k];
        for (size_t j = 0; j < blk; ++j) R[e * blk + j] += tmp[j];
    }
    if (visc) {
        for (int k = 0; k < m->nbf; ++k) {
            int tag = m->bfaces[3 * k + 2];
            if (tag < 0 || tag >= MAX_TAGS || !m->bc[tag].set) continue;
            orc_boundary_face_residual(m, ph, k, u, 1, tmp);
            int e = m->bfaces[3 * k];
            for (size_t j = 0; j < blk; ++j) R[e * blk + j] += tmp[j];
        }
    }
    return err;
}

/* TimeDependentWeakFormulation::compute_mass_integral, weak_formulation_base.cpp:198-217 */
int orc_mass_matrix(const orc_mesh* m, int e, double* M) {
    int np = m->np, nq = m->nq;
    memset(M, 0, sizeof(double) * np * np);
    for (int q = 0; q < nq; ++q) {
        double w = m->qw[q] * fabs(m->jdet[(size_t)e * nq + q]);
        const double* ph = m->phi_vol + q * np;
        for (int i = 0; i < np; ++i)
            for (int j = 0; j < np; ++j) M[i * np + j] += w * (ph[i] * ph[j]);
    }
    return 0;
}

/* Dense inverse by LU with partial pivoting (what Eigen's MatrixXd::inverse() does for
 * dynamic sizes), used by compute_mass_matrix_inverse_blocks,
 * compressible_solver_base.cpp:41-52 */
static int lu_inverse(int n, const double* A, double* Ainv) {
    double LU[64 * 64];
    int piv[64];
    memcpy(LU, A, sizeof(double) * n * n);
    for (int i = 0; i < n; ++i) piv[i] = i;
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(LU[k * n + k]);
        for (int r = k + 1; r < n; ++r)
            if (fabs(LU[r * n + k]) > best) { best = fabs(LU[r * n + k]); p = r; }
        if (best == 0.0) return -1;
        if (p != k) {
            for (int c = 0; c < n; ++c) {
                double t = LU[k * n + c]; LU[k * n + c] = LU[p * n + c]; LU[p * n + c] = t;
            }
            int t = piv[k]; piv[k] = piv[p]; piv[p] = t;
        }
        for (int r = k + 1; r < n; ++r) {
            double l = LU[r * n + k] / LU[k * n + k];
            LU[r * n + k] = l;
            for (int c = k + 1; c < n; ++c) LU[r * n + c] -= l * LU[k * n + c];
        }
    }
    for (int col = 0; col < n; ++col) {
        double y[64];
        for (int i = 0; i < n; ++i) {
            double s = (piv[i] == col) ? 1.0 : 0.0;
            for (int j = 0; j < i; ++j) s -= LU[i * n + j] * y[j];
            y[i] = s;
        }
        for (int i = n - 1; i >= 0; --i) {
            double s = y[i];
            for (int j = i + 1; j < n; ++j) s -= LU[i * n + j] * Ainv[j * n + col];
            Ainv[i * n + col] = s / LU[i * n + i];
        }
    }
    return 0;
}

int orc_compute_mass_inverse(orc_mesh* m) {
    int np = m->np, ne = m->ne;
    if (!m->space_ready) return -1;
    free(m->minv);
    m->minv = (double*)malloc(sizeof(double) * (size_t)ne * np * np);
    int err = 0;
#pragma omp parallel for num_threads(g_threads) reduction(| : err) schedule(static)
    for (int e = 0; e < ne; ++e) {
        double M[64 * 64];
        orc_mass_matrix(m, e, M);
        err |= lu_inverse(np, M, m->minv + (size_t)e * np * np);
    }
    return err;
}

/* CompressibleDGSolverBase::apply_mass_inv, compressible_solver_base.cpp:54-61 */
int orc_apply_mass_inv(const orc_mesh* m, const double* in, double* out) {
    int np = m->np, ne = m->ne;
    if (!m->minv) return -1;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int e = 0; e < ne; ++e) {
        const double* Mi = m->minv + (size_t)e * np * np;
        const double* a = in + (size_t)e * np * NV;
        double* o = out + (size_t)e * np * NV;
        for (int i = 0; i < np; ++i)
            for (int v = 0; v < NV; ++v) {
                double s = 0.0;
                for (int k = 0; k < np; ++k) s += Mi[i * np + k] * a[k * NV + v];
                o[i * NV + v] = s;
            }
    }
    return 0;
}

/* rhs_func = apply_mass_inv(assemble_residual(u)), compressible_solver_base.cpp:106-112 */
int orc_rhs(const orc_mesh* m, const orc_physics* ph, const double* u, double* du) {
    size_t n = (size_t)m->ne * m->np * NV;
    double* R = (double*)malloc(sizeof(double) * n);
    int err = orc_assemble_residual(m, ph, u, R);
    if (!err) err = orc_apply_mass_inv(m, R, du);
    free(R);
    return err;
}

/* SSP_RK::step_rk3, time_stepping.hpp:39-55 with add_scaled/scale :59-85 */
int orc_rk3_step(const orc_mesh* m, const orc_physics* ph, double* u, double dt) {
    size_t n = (size_t)m->ne * m->np * NV;
    double* k = (double*)malloc(sizeof(double) * n);
    double* u1 = (double*)malloc(sizeof(double) * n);
    double* u2 = (double*)malloc(sizeof(double) * n);
    int err = orc_rhs(m, ph, u, k);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (size_t j = 0; j < n; ++j) u1[j] = u[j] + dt * k[j];
    err |= orc_rhs(m, ph, u1, k);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (size_t j = 0; j < n; ++j) {
        double t = u1[j] + dt * k[j];
        double s = 0.75 * u[j];
        u2[j] = s + 0.25 * t;
    }
    err |= orc_rhs(m, ph, u2, k);
    const double a = 1.0 / 3.0, b = 2.0 / 3.0;
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (size_t j = 0; j < n; ++j) {
        double t = u2[j] + dt * k[j];
        double s = a * u[j];
        u[j] = s + b * t;
    }
    free(k); free(u1); free(u2);
    return err;
}

/* CompressibleDGSolverBase::compute_max_cfl, compressible_solver_base.cpp:114-170 */
double orc_max_cfl(const orc_mesh* m, double gamma, const double* u, double dt) {
    int np = m->np, nq = m->nq;
    double max_cfl = 0.0;
    for (int e = 0; e < m->ne; ++e) {
        double V[8];
        elem_verts(m, e, V);
        double h = 1.79769313486231570815e308;
        for (int i = 0; i < m->nvpe; ++i)
            for (int j = i + 1; j < m->nvpe; ++j) {
                double dx = V[2 * i] - V[2 * j], dy = V[2 * i + 1] - V[2 * j + 1];
                double d = sqrt(dx * dx + dy * dy);
                h = fmin(h, d);
            }
        double mws = 0.0;
        const double* ue = UE(u, e, np);
        for (int q = 0; q < nq; ++q) {
            double U[4] = {0, 0, 0, 0};
            for (int i = 0; i < np; ++i)
                for (int v = 0; v < NV; ++v) U[v] += m->phi_vol[q * np + i] * ue[i * NV + v];
            double rho = U[0];
            if (rho <= 0.0 || !isfinite(rho)) return INFINITY;
            double uu = U[1] / rho, vv = U[2] / rho;
            double kin = 0.5 * (uu * uu + vv * vv);
            double p = (gamma - 1.0) * (U[3] - rho * kin);
            if (p <= 0.0 || !isfinite(p)) return INFINITY;
            double c = sqrt(fmax(gamma * p / rho, 0.0));
            double ws = sqrt(uu * uu + vv * vv) + c;
            mws = fmax(mws, ws);
        }
        max_cfl = fmax(max_cfl, dt * mws / h);
    }
    return max_cfl;
}

/* CompressibleDGSolverBase::compute_density_range, compressible_solver_base.cpp:172-199 */
void orc_density_range(const orc_mesh* m, const double* u, double* rmin, double* rmax) {
    int np = m->np, nq = m->nq;
    double lo = INFINITY, hi = -1.79769313486231570815e308;
    for (int e = 0; e < m->ne; ++e) {
        const double* ue = UE(u, e, np);
        for (int q = 0; q < nq; ++q) {
            double rho = 0.0;
            for (int i = 0; i < np; ++i) rho += m->phi_vol[q * np + i] * ue[i * NV];
            if (!isfinite(rho)) continue;
            lo = fmin(lo, rho);
            hi = fmax(hi, rho);
        }
    }
    if (!isfinite(lo) || !isfinite(hi)) { lo = NAN; hi = NAN; }
    *rmin = lo;
    *rmax = hi;
}

/* CompressibleDGSolverBase::project_initial_condition, compressible_solver_base.cpp:63-104;
 * Uq holds the initial condition evaluated at orc_mesh_quad_points. */
int orc_project(const orc_mesh* m, const double* Uq, double* u) {
    int np = m->np, nq = m->nq, ne = m->ne;
    size_t n = (size_t)ne * np * NV;
    double* F = (double*)calloc(n, sizeof(double));
    for (int e = 0; e < ne; ++e) {
        double* Fe = F + (size_t)e * np * NV;
        for (int q = 0; q < nq; ++q) {
            double w = m->qw[q] * fabs(m->jdet[(size_t)e * nq + q]);
            const double* U = Uq + ((size_t)e * nq + q) * NV;
            for (int i = 0; i < np; ++i) {
                double s = w * m->phi_vol[q * np + i];
                for (int v = 0; v < NV; ++v) Fe[i * NV + v] += s * U[v];
            }
        }
    }
    int err = orc_apply_mass_inv(m, F, u);
    free(F);
    return err;
}
