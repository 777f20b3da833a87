// Device-side set-up: the pairing of element faces by their vertex pair (DGMesh's
// build_face_connectivity, src/core/mesh.cpp:312-359) and the element geometry
// (DGSpace::compute_element_data / compute_face_data, src/core/space.cpp:69-171, with
// GeometricMapping::compute_mapping, src/reference/mapping.cpp:22-50), on the GPU.
//
// The pairing sorts the face slots by their packed vertex-pair key with a stable radix sort (CUB,
// part of the CUDA toolkit; set-up only), so equal keys stay in slot order and the first two slots
// of a key become neighbours: the table the host's own stable radix sort builds, entry for entry.
// The geometry kernels compute, per element, what dgx_host.cpp's build_geometry computes, with
// every FP64 operation written as an explicitly rounded one (no contraction): A = inverse(J_T),
// |det J_T|, the shortest vertex distance, the volume points in physical space, and per face the
// outward normal and length -- the L side's for both sides of an interior face (the R side
// recomputes the L side's from the L element's vertices) -- so the records equal the host's bit
// for bit (the host side is compiled without floating-point contraction too).
#include <cub/device/device_radix_sort.cuh>

#include <cstdint>

#include "dgx_internal.h"

namespace dgx {

namespace {

__global__ void face_keys_kernel(int ne, int K, const int* __restrict__ elems, uint64_t nv, uint64_t* key,
                                 int* slot) {
    const size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (s >= (size_t)ne * K) return;
    const size_t e = s / K;
    const int f = (int)(s - e * K);
    const int v1 = elems[e * K + f], v2 = elems[e * K + (f + 1) % K];
    key[s] = (uint64_t)min(v1, v2) * nv + (uint64_t)max(v1, v2);
    slot[s] = (int)s;
}

// the first two slots of each run of equal keys become neighbours
__global__ void pair_slots_kernel(size_t ns, int K, const uint64_t* __restrict__ key, const int* __restrict__ slot,
                                  int* nbr) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i + 1 >= ns) return;
    if (key[i + 1] != key[i] || (i > 0 && key[i - 1] == key[i])) return;
    const int s1 = slot[i], s2 = slot[i + 1];
    nbr[2 * (size_t)s1] = s2 / K;
    nbr[2 * (size_t)s1 + 1] = s2 % K;
    nbr[2 * (size_t)s2] = s1 / K;
    nbr[2 * (size_t)s2 + 1] = s1 % K;
}

// ---- geometry, every operation rounded as the host's (no fused multiply-adds)
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

template <int NV>
__device__ __forceinline__ void load_verts(const double* __restrict__ verts, const int* __restrict__ elems, int e,
                                           double (&V)[2 * NV]) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const int v = elems[(size_t)NV * e + k];
        V[2 * k] = verts[2 * (size_t)v];
        V[2 * k + 1] = verts[2 * (size_t)v + 1];
    }
}

// face_geom (dgx_host.cpp): outward normal and length of face f, from vertex f to vertex f + 1
template <int NV>
__device__ __forceinline__ bool face_geom_d(const double (&V)[2 * NV], int f, double& nx, double& ny, double& len) {
    const int a = f, b = (f + 1) % NV;
    const double tx = sub(V[2 * b], V[2 * a]), ty = sub(V[2 * b + 1], V[2 * a + 1]);
    len = __dsqrt_rn(add(mul(tx, tx), mul(ty, ty)));
    if (len < 1e-14) return false;
    nx = __ddiv_rn(ty, len);
    ny = __ddiv_rn(-tx, len);
    double cx = 0.0, cy = 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        cx = add(cx, V[2 * k]);
        cy = add(cy, V[2 * k + 1]);
    }
    cx = __ddiv_rn(cx, (double)NV);
    cy = __ddiv_rn(cy, (double)NV);
    const double mx = mul(0.5, add(V[2 * a], V[2 * b])), my = mul(0.5, add(V[2 * a + 1], V[2 * b + 1]));
    if (add(mul(nx, sub(mx, cx)), mul(ny, sub(my, cy))) < 0) {
        nx = -nx;
        ny = -ny;
    }
    return true;
}

template <int NV>
__device__ __forceinline__ double shortest_vertex_distance_d(const double (&V)[2 * NV]) {
    double h = 1.7976931348623157e308;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int j = i + 1; j < NV; ++j) {
            const double dx = sub(V[2 * i], V[2 * j]), dy = sub(V[2 * i + 1], V[2 * j + 1]);
            h = fmin(h, __dsqrt_rn(add(mul(dx, dx), mul(dy, dy))));
        }
    return h;
}

// the face's normal and length as the element's record holds them: its own for an L side or a
// boundary face, minus the L side's normal and the L side's length for an R side
template <int NV, class Conn>
__device__ __forceinline__ bool face_record(const double* __restrict__ verts, const int* __restrict__ elems,
                                            const double (&V)[2 * NV], const Conn& C, int f, double& nx, double& ny,
                                            double& len) {
    const int nb = C.nbr[f];
    const int fl = (C.flags >> (4 * f)) & 15;
    if (nb >= 0 && !(fl & 8)) {  // R side: the L side's face
        double VL[2 * NV];
        load_verts<NV>(verts, elems, nb, VL);
        if (!face_geom_d<NV>(VL, fl & 3, nx, ny, len)) return false;
        nx = -nx;
        ny = -ny;
        return true;
    }
    return face_geom_d<NV>(V, f, nx, ny, len);
}

}  // namespace

int device_face_pairs(int ne, int K, const int* elems_host, long long nv, int* nbr_host) {
    const size_t ns = (size_t)ne * K;
    if (ns == 0) return 0;
    if (ns > 0x7fffffffu) return -1;
    cudaStream_t s = nullptr;
    int* d_elems = nullptr;
    uint64_t *d_key = nullptr, *d_key2 = nullptr;
    int *d_slot = nullptr, *d_slot2 = nullptr, *d_nbr = nullptr;
    void* d_tmp = nullptr;
    size_t tmp = 0;
    int end_bit = 1;
    const unsigned long long kmax = (unsigned long long)nv * (unsigned long long)nv;
    while (end_bit < 64 && (kmax >> end_bit) != 0) ++end_bit;
    int rc = -1;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
        cudaMalloc((void**)&d_elems, ns * sizeof(int)) == cudaSuccess &&
        cudaMalloc((void**)&d_key, ns * sizeof(uint64_t)) == cudaSuccess &&
        cudaMalloc((void**)&d_key2, ns * sizeof(uint64_t)) == cudaSuccess &&
        cudaMalloc((void**)&d_slot, ns * sizeof(int)) == cudaSuccess &&
        cudaMalloc((void**)&d_slot2, ns * sizeof(int)) == cudaSuccess &&
        cudaMalloc((void**)&d_nbr, 2 * ns * sizeof(int)) == cudaSuccess &&
        cub::DeviceRadixSort::SortPairs(nullptr, tmp, d_key, d_key2, d_slot, d_slot2, (int)ns, 0, end_bit, s) ==
            cudaSuccess &&
        cudaMalloc(&d_tmp, tmp ? tmp : 16) == cudaSuccess &&
        cudaMemcpyAsync(d_elems, elems_host, ns * sizeof(int), cudaMemcpyHostToDevice, s) == cudaSuccess &&
        cudaMemsetAsync(d_nbr, 0xff, 2 * ns * sizeof(int), s) == cudaSuccess) {
        const unsigned blocks = (unsigned)((ns + 255) / 256);
        face_keys_kernel<<<blocks, 256, 0, s>>>(ne, K, d_elems, (uint64_t)nv, d_key, d_slot);
        if (cudaGetLastError() == cudaSuccess &&
            cub::DeviceRadixSort::SortPairs(d_tmp, tmp, d_key, d_key2, d_slot, d_slot2, (int)ns, 0, end_bit, s) ==
                cudaSuccess) {
            pair_slots_kernel<<<blocks, 256, 0, s>>>(ns, K, d_key2, d_slot2, d_nbr);
            if (cudaGetLastError() == cudaSuccess &&
                cudaMemcpyAsync(nbr_host, d_nbr, 2 * ns * sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                cudaStreamSynchronize(s) == cudaSuccess)
                rc = 0;
        }
    }
    if (rc) last_launch_error() = cudaGetLastError();
    cudaFree(d_tmp);
    cudaFree(d_nbr);
    cudaFree(d_slot2);
    cudaFree(d_slot);
    cudaFree(d_key2);
    cudaFree(d_key);
    cudaFree(d_elems);
    if (s) cudaStreamDestroy(s);
    return rc;
}

namespace {

struct SetupPoints {
    int nq, nfq;
    double qp[OPS_MAX_NQ][2];
    double fxi[4][OPS_MAX_NFQ][2];
};

// err bits: 1 singular Jacobian, 2 degenerate edge
__global__ void tri_geometry_kernel(int ne, const double* __restrict__ verts, const int* __restrict__ elems,
                                    const ElemConn* __restrict__ conn, const __grid_constant__ SetupPoints pts,
                                    ElemGeom* geom, ElemGeomF* geomf, double* xq, int* err) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double V[6];
    load_verts<3>(verts, elems, e, V);
    ElemGeom g;
    for (int k = 0; k < 2; ++k) g.pad[k] = 0.0;
    const double J00 = sub(V[2], V[0]), J01 = sub(V[3], V[1]);
    const double J10 = sub(V[4], V[0]), J11 = sub(V[5], V[1]);
    const double det = sub(mul(J00, J11), mul(J10, J01));
    if (fabs(det) < 1e-12) atomicOr(err, 1);
    const double inv = __ddiv_rn(1.0, det);
    g.A[0] = mul(J11, inv);
    g.A[2] = mul(-J10, inv);
    g.A[1] = mul(-J01, inv);
    g.A[3] = mul(J00, inv);
    g.detJ = fabs(det);
    g.pad[0] = shortest_vertex_distance_d<3>(V);
    const ElemConn C = conn[e];
    for (int f = 0; f < 3; ++f) {
        double nx = 0.0, ny = 0.0, len = 0.0;
        if (!face_record<3>(verts, elems, V, C, f, nx, ny, len)) atomicOr(err, 2);
        g.n[f][0] = nx;
        g.n[f][1] = ny;
        g.h[f] = len;
    }
    geom[e] = g;
    if (geomf) {
        ElemGeomF h;
        for (int k = 0; k < 4; ++k) h.A[k] = __double2float_rn(g.A[k]);
        h.detJ = __double2float_rn(g.detJ);
        for (int f = 0; f < 3; ++f) {
            h.h[f] = __double2float_rn(g.h[f]);
            h.n[f][0] = __double2float_rn(g.n[f][0]);
            h.n[f][1] = __double2float_rn(g.n[f][1]);
        }
        h.hmin = __double2float_rn(g.pad[0]);
        h.pad = 0.0f;  // instance 0
        geomf[e] = h;
    }
    for (int q = 0; q < pts.nq; ++q) {  // map_to_physical: V^T N
        const double xi = pts.qp[q][0], eta = pts.qp[q][1];
        const double N0 = sub(sub(1.0, xi), eta);
        xq[((size_t)e * pts.nq + q) * 2] = add(add(mul(N0, V[0]), mul(xi, V[2])), mul(eta, V[4]));
        xq[((size_t)e * pts.nq + q) * 2 + 1] = add(add(mul(N0, V[1]), mul(xi, V[3])), mul(eta, V[5]));
    }
}

__global__ void quad_geometry_kernel(int ne, const double* __restrict__ verts, const int* __restrict__ elems,
                                     const QuadConn* __restrict__ conn, const __grid_constant__ SetupPoints pts,
                                     QuadGeom* geom, QuadGeomF* geomf, double* xq, int* err) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double V[8];
    load_verts<4>(verts, elems, e, V);
    QuadGeom g;
    for (int k = 0; k < 5; ++k) g.pad[k] = 0.0;
    for (int c = 0; c < 2; ++c) {
        const double x0 = V[c], x1 = V[2 + c], x2 = V[4 + c], x3 = V[6 + c];
        double* j = c == 0 ? g.jx : g.jy;
        j[0] = mul(0.25, add(sub(x1, x0), sub(x2, x3)));
        j[1] = mul(0.25, add(sub(x3, x0), sub(x2, x1)));
        j[2] = mul(0.25, add(sub(x0, x1), sub(x2, x3)));
    }
    auto det_at = [&](double xi, double eta) {
        const double J00 = add(g.jx[0], mul(g.jx[2], eta)), J01 = add(g.jy[0], mul(g.jy[2], eta));
        const double J10 = add(g.jx[1], mul(g.jx[2], xi)), J11 = add(g.jy[1], mul(g.jy[2], xi));
        return sub(mul(J00, J11), mul(J10, J01));
    };
    bool singular = false;
    for (int q = 0; q < pts.nq; ++q) singular |= fabs(det_at(pts.qp[q][0], pts.qp[q][1])) < 1e-12;
    for (int f = 0; f < 4; ++f)
        for (int q = 0; q < pts.nfq; ++q) singular |= fabs(det_at(pts.fxi[f][q][0], pts.fxi[f][q][1])) < 1e-12;
    if (singular) atomicOr(err, 1);
    g.hmin = shortest_vertex_distance_d<4>(V);
    const QuadConn C = conn[e];
    for (int f = 0; f < 4; ++f) {
        double nx = 0.0, ny = 0.0, len = 0.0;
        if (!face_record<4>(verts, elems, V, C, f, nx, ny, len)) atomicOr(err, 2);
        g.n[f][0] = nx;
        g.n[f][1] = ny;
        g.h[f] = len;
    }
    geom[e] = g;
    if (geomf) {
        QuadGeomF h;
        for (int k = 0; k < 3; ++k) {
            h.jx[k] = __double2float_rn(g.jx[k]);
            h.jy[k] = __double2float_rn(g.jy[k]);
        }
        for (int f = 0; f < 4; ++f) {
            h.h[f] = __double2float_rn(g.h[f]);
            h.n[f][0] = __double2float_rn(g.n[f][0]);
            h.n[f][1] = __double2float_rn(g.n[f][1]);
        }
        h.hmin = __double2float_rn(g.hmin);
        for (int k = 0; k < 5; ++k) h.pad[k] = 0.0f;
        geomf[e] = h;
    }
    for (int q = 0; q < pts.nq; ++q) {  // map_to_physical: V^T N (ReferenceQuad shape functions)
        const double xi = pts.qp[q][0], eta = pts.qp[q][1];
        const double N[4] = {mul(mul(0.25, sub(1.0, xi)), sub(1.0, eta)), mul(mul(0.25, add(1.0, xi)), sub(1.0, eta)),
                             mul(mul(0.25, add(1.0, xi)), add(1.0, eta)), mul(mul(0.25, sub(1.0, xi)), add(1.0, eta))};
        double x = 0.0, y = 0.0;
        for (int k = 0; k < 4; ++k) {
            x = add(x, mul(N[k], V[2 * k]));
            y = add(y, mul(N[k], V[2 * k + 1]));
        }
        xq[((size_t)e * pts.nq + q) * 2] = x;
        xq[((size_t)e * pts.nq + q) * 2 + 1] = y;
    }
}

}  // namespace

int launch_device_geometry(int ne, int nvpe, const OpsHost& ops, const double* d_verts, const int* d_elems,
                           const void* d_conn, void* d_geom, void* d_geomf, double* d_xq, int* d_err,
                           cudaStream_t s) {
    if (ne == 0) return 0;
    SetupPoints pts{};
    pts.nq = ops.nq;
    pts.nfq = ops.nfq;
    for (int q = 0; q < ops.nq; ++q) {
        pts.qp[q][0] = ops.qp[q][0];
        pts.qp[q][1] = ops.qp[q][1];
    }
    for (int f = 0; f < 4; ++f)
        for (int q = 0; q < ops.nfq; ++q) {
            pts.fxi[f][q][0] = ops.fxi[f][q][0];
            pts.fxi[f][q][1] = ops.fxi[f][q][1];
        }
    const unsigned blocks = (unsigned)((ne + 127) / 128);
    if (nvpe == 4)
        quad_geometry_kernel<<<blocks, 128, 0, s>>>(ne, d_verts, d_elems, static_cast<const QuadConn*>(d_conn), pts,
                                                    static_cast<QuadGeom*>(d_geom), static_cast<QuadGeomF*>(d_geomf),
                                                    d_xq, d_err);
    else
        tri_geometry_kernel<<<blocks, 128, 0, s>>>(ne, d_verts, d_elems, static_cast<const ElemConn*>(d_conn), pts,
                                                   static_cast<ElemGeom*>(d_geom), static_cast<ElemGeomF*>(d_geomf),
                                                   d_xq, d_err);
    return launch_status();
}

}  // namespace dgx
