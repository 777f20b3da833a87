"""ctypes front end of the CPU oracle (``dg_oracle.c``).

TEST INFRASTRUCTURE ONLY: the parity checker for the GPU path and the timed CPU
baseline.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs
use it.  The oracle restates dgfem's residual-and-update path in FP64; see
``dg_oracle.h`` for the per-function citations and how it is pinned.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

MONOMIAL, DUBINER, LEGENDRE = 0, 1, 2  # LEGENDRE: the quad basis
FAR_FIELD, SLIP_WALL, NO_SLIP_WALL, PERIODIC = 0, 1, 2, 3

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
BCFN = C.CFUNCTYPE(None, C.c_double, C.c_double, C.POINTER(C.c_double), C.c_void_p)


class Physics(C.Structure):
    _fields_ = [("gamma", C.c_double), ("viscous", C.c_int), ("mu", C.c_double),
                ("prandtl", C.c_double), ("sigma0", C.c_double)]


def euler(gamma=1.4):
    return Physics(gamma, 0, 0.0, 0.0, 0.0)


def navier_stokes(gamma=1.4, mu=1.0e-3, prandtl=0.72, sigma0=5.0):
    return Physics(gamma, 1, mu, prandtl, sigma0)


def build():
    """Compile the oracle (make); returns the library path."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.orc_tri_rule.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.POINTER(C.c_double)),
                                   C.POINTER(C.POINTER(C.c_double))]
        L.orc_gl_rule.argtypes = [C.c_int, C.POINTER(C.POINTER(C.c_double)),
                                  C.POINTER(C.POINTER(C.c_double))]
        L.orc_basis_eval.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.orc_basis_grad.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.orc_compute_mapping.argtypes = [_dp, C.c_double, C.c_double, _dp, _dp, _dp]
        L.orc_map_face_point.argtypes = [C.c_int, C.c_double, _dp]
        L.orc_compute_mapping_nv.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp, _dp, _dp]
        L.orc_map_face_point_nv.argtypes = [C.c_int, C.c_int, C.c_double, _dp]
        L.orc_mesh_create_nv.restype = C.c_void_p
        L.orc_mesh_create_nv.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, C.c_int, _ip]
        L.orc_mesh_create.restype = C.c_void_p
        L.orc_mesh_create.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip]
        L.orc_mesh_destroy.argtypes = [C.c_void_p]
        L.orc_mesh_set_periodic.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.orc_mesh_init_space.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_mesh_rebuild_faces.argtypes = [C.c_void_p]
        L.orc_mesh_n_interior_faces.argtypes = [C.c_void_p]
        L.orc_mesh_n_boundary_faces.argtypes = [C.c_void_p]
        L.orc_mesh_interior_faces.argtypes = [C.c_void_p, _ip]
        L.orc_mesh_boundary_faces.argtypes = [C.c_void_p, _ip]
        L.orc_mesh_neighbors.argtypes = [C.c_void_p, _ip]
        L.orc_mesh_set_bc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
        L.orc_mesh_space_dims.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]
        L.orc_mesh_element_data.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.orc_mesh_face_data.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_space_tables.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_mesh_quad_points.argtypes = [C.c_void_p, _dp]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_rusanov.argtypes = [C.c_double, _dp, _dp, _dp, _dp]
        L.orc_viscous_flux.argtypes = [C.POINTER(Physics), _dp, _dp, _dp, _dp]
        L.orc_penalty.restype = C.c_double
        L.orc_penalty.argtypes = [C.POINTER(Physics), C.c_int, C.c_double]
        for name in ("orc_volume_residual", "orc_viscous_volume_residual"):
            getattr(L, name).argtypes = [C.c_void_p, C.POINTER(Physics), C.c_int, _dp, _dp]
        L.orc_interior_face_residual.argtypes = [C.c_void_p, C.POINTER(Physics), C.c_int, _dp,
                                                 C.c_int, _dp, _dp]
        L.orc_boundary_face_residual.argtypes = [C.c_void_p, C.POINTER(Physics), C.c_int, _dp,
                                                 C.c_int, _dp]
        L.orc_assemble_residual.argtypes = [C.c_void_p, C.POINTER(Physics), _dp, _dp]
        L.orc_mass_matrix.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_compute_mass_inverse.argtypes = [C.c_void_p]
        L.orc_apply_mass_inv.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_rhs.argtypes = [C.c_void_p, C.POINTER(Physics), _dp, _dp]
        L.orc_rk3_step.argtypes = [C.c_void_p, C.POINTER(Physics), _dp, C.c_double]
        L.orc_max_cfl.restype = C.c_double
        L.orc_max_cfl.argtypes = [C.c_void_p, C.c_double, _dp, C.c_double]
        L.orc_density_range.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
        L.orc_project.argtypes = [C.c_void_p, _dp, _dp]
        _lib = L
    return _lib


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def tri_rule(order):
    n = C.c_int()
    p = C.POINTER(C.c_double)()
    w = C.POINTER(C.c_double)()
    if lib().orc_tri_rule(order, C.byref(n), C.byref(p), C.byref(w)):
        raise ValueError(order)
    return (np.ctypeslib.as_array(p, (n.value, 2)).copy(), np.ctypeslib.as_array(w, (n.value,)).copy())


def gl_rule(n):
    p = C.POINTER(C.c_double)()
    w = C.POINTER(C.c_double)()
    if lib().orc_gl_rule(n, C.byref(p), C.byref(w)):
        raise ValueError(n)
    return np.ctypeslib.as_array(p, (n,)).copy(), np.ctypeslib.as_array(w, (n,)).copy()


def n_basis(p, basis=MONOMIAL):
    return (p + 1) * (p + 1) if basis == LEGENDRE else (p + 1) * (p + 2) // 2


def basis_eval(basis, p, x, y):
    out = np.zeros(n_basis(p, basis))
    lib().orc_basis_eval(basis, p, x, y, out)
    return out


def basis_grad(basis, p, x, y):
    out = np.zeros((n_basis(p, basis), 2))
    lib().orc_basis_grad(basis, p, x, y, out)
    return out


def compute_mapping(verts, xi, eta):
    """Returns (x_phys, J_det, dxi_dx) or raises RuntimeError on a singular Jacobian.
    verts: 3 (triangle) or 4 (quad) vertices."""
    V = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1, 2)
    x = np.zeros(2)
    d = np.zeros(1)
    A = np.zeros((2, 2))
    if lib().orc_compute_mapping_nv(len(V), np.ascontiguousarray(V), xi, eta, x, d, A):
        raise RuntimeError("Singular Jacobian matrix")
    return x, d[0], A


def map_face_point(face, s, nv=3):
    out = np.zeros(2)
    lib().orc_map_face_point_nv(nv, face, s, out)
    return out


def rusanov(gamma, UL, UR, n):
    H = np.zeros(4)
    lib().orc_rusanov(gamma, np.ascontiguousarray(UL, np.float64), np.ascontiguousarray(UR, np.float64),
                      np.ascontiguousarray(n, np.float64), H)
    return H


def viscous_flux(phys, U, gradU):
    Fv = np.zeros(4)
    Gv = np.zeros(4)
    lib().orc_viscous_flux(C.byref(phys), np.ascontiguousarray(U, np.float64),
                           np.ascontiguousarray(gradU, np.float64).reshape(4, 2), Fv, Gv)
    return Fv, Gv


def penalty(phys, p, h):
    return lib().orc_penalty(C.byref(phys), p, h)


class OracleMesh:
    """DGMesh + DGSpace + CompressibleDGSolverBase state, restated on the CPU."""

    def __init__(self, vertices, elements, boundary_edges=None, order=1, basis=MONOMIAL,
                 periodic=()):
        L = lib()
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 2)
        nvpe = np.asarray(elements).shape[-1]
        self.nvpe = nvpe
        self.elements = np.ascontiguousarray(elements, dtype=np.int32).reshape(-1, nvpe)
        be = np.zeros((0, 3), np.int32) if boundary_edges is None else \
            np.ascontiguousarray(boundary_edges, dtype=np.int32).reshape(-1, 3)
        # dgfem's boundary_edges is a std::map keyed by tag: iterate tags in ascending order
        be = be[np.argsort(be[:, 0], kind="stable")] if len(be) else be
        self.h = L.orc_mesh_create_nv(nvpe, len(self.vertices), self.vertices, len(self.elements),
                                      self.elements, len(be), np.ascontiguousarray(be))
        self.order = order
        self.basis = basis
        rc = L.orc_mesh_init_space(self.h, order, basis)
        if rc:
            raise RuntimeError(f"init_space failed ({rc})")
        for t1, t2, match_y in periodic:
            if L.orc_mesh_set_periodic(self.h, t1, t2, int(match_y)):
                raise RuntimeError("Cannot set periodic boundaries")
        np_, nq, nfq = C.c_int(), C.c_int(), C.c_int()
        L.orc_mesh_space_dims(self.h, C.byref(np_), C.byref(nq), C.byref(nfq))
        self.np, self.nq, self.nfq = np_.value, nq.value, nfq.value
        self.ne = len(self.elements)
        self._bc_keep = []
        self._minv = False

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None

    # ---- mesh queries
    def interior_faces(self):
        n = lib().orc_mesh_n_interior_faces(self.h)
        out = np.zeros((n, 5), np.int32)
        if n:
            lib().orc_mesh_interior_faces(self.h, out)
        return out

    def boundary_faces(self):
        n = lib().orc_mesh_n_boundary_faces(self.h)
        out = np.zeros((n, 3), np.int32)
        if n:
            lib().orc_mesh_boundary_faces(self.h, out)
        return out

    def neighbors(self):
        out = np.zeros((self.ne, self.nvpe, 2), np.int32)
        lib().orc_mesh_neighbors(self.h, out)
        return out

    def element_data(self, e):
        J = np.zeros(self.nq)
        D = np.zeros((self.nq * self.np, 2))
        lib().orc_mesh_element_data(self.h, e, J, D)
        return {"J_det_vol": J, "dphi_dx_vol": D}

    def face_data(self, e, f):
        n = np.zeros(2)
        ln = np.zeros(1)
        qp = np.zeros(2 * self.nfq)
        D = np.zeros((self.nfq * self.np, 2))
        lib().orc_mesh_face_data(self.h, e, f, n, ln, qp, D)
        return {"normal": n, "length": ln[0], "quad_points": qp, "dphi_dx_face": D}

    def tables(self):
        pv = np.zeros((self.nq, self.np))
        pf = np.zeros((self.nvpe, self.nfq, self.np))
        vw = np.zeros(self.nq)
        fw = np.zeros(self.nfq)
        lib().orc_space_tables(self.h, pv, pf, vw, fw)
        return {"phi_vol": pv, "phi_face": pf, "vol_w": vw, "face_w": fw}

    def quad_points(self):
        out = np.zeros((self.ne, self.nq, 2))
        lib().orc_mesh_quad_points(self.h, out)
        return out

    def set_bc(self, tag, bc_type, value=None, fn=None):
        """Constant value, or fn(x, y) -> 4 values (kept alive by this object)."""
        v = None if value is None else np.ascontiguousarray(value, np.float64)
        cb = None
        if fn is not None:
            def _cb(x, y, out, _u):
                r = fn(x, y)
                for i in range(4):
                    out[i] = float(r[i])
            cb = BCFN(_cb)
            self._bc_keep.append(cb)
        if v is not None:
            self._bc_keep.append(v)
        rc = lib().orc_mesh_set_bc(self.h, tag, bc_type,
                                   None if v is None else v.ctypes.data_as(C.c_void_p),
                                   None if cb is None else C.cast(cb, C.c_void_p), None)
        if rc:
            raise ValueError(tag)

    def rebuild_faces(self):
        lib().orc_mesh_rebuild_faces(self.h)

    # ---- physics
    def _state(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(self.ne, self.np, 4)
        return u

    def residual(self, phys, u):
        u = self._state(u)
        R = np.zeros_like(u)
        rc = lib().orc_assemble_residual(self.h, C.byref(phys), u, R)
        if rc:
            raise RuntimeError(f"assemble_residual failed ({rc})")
        return R

    def volume_residual(self, phys, e, u, viscous=False):
        u = self._state(u)
        R = np.zeros((self.np, 4))
        f = lib().orc_viscous_volume_residual if viscous else lib().orc_volume_residual
        f(self.h, C.byref(phys), e, u, R)
        return R

    def interior_face_residual(self, phys, k, u, viscous=False):
        u = self._state(u)
        RL = np.zeros((self.np, 4))
        RR = np.zeros((self.np, 4))
        lib().orc_interior_face_residual(self.h, C.byref(phys), k, u, int(viscous), RL, RR)
        return RL, RR

    def boundary_face_residual(self, phys, k, u, viscous=False):
        u = self._state(u)
        R = np.zeros((self.np, 4))
        rc = lib().orc_boundary_face_residual(self.h, C.byref(phys), k, u, int(viscous), R)
        if rc:
            raise RuntimeError(f"boundary_face_residual failed ({rc})")
        return R

    def mass_matrix(self, e):
        M = np.zeros((self.np, self.np))
        lib().orc_mass_matrix(self.h, e, M)
        return M

    def _ensure_minv(self):
        if not self._minv:
            if lib().orc_compute_mass_inverse(self.h):
                raise RuntimeError("mass inverse failed")
            self._minv = True

    def apply_mass_inv(self, R):
        self._ensure_minv()
        R = self._state(R)
        out = np.zeros_like(R)
        lib().orc_apply_mass_inv(self.h, R, out)
        return out

    def rhs(self, phys, u):
        self._ensure_minv()
        u = self._state(u)
        out = np.zeros_like(u)
        if lib().orc_rhs(self.h, C.byref(phys), u, out):
            raise RuntimeError("rhs failed")
        return out

    def rk3_step(self, phys, u, dt, n_steps=1):
        self._ensure_minv()
        u = np.array(self._state(u), copy=True)
        for _ in range(n_steps):
            if lib().orc_rk3_step(self.h, C.byref(phys), u, dt):
                raise RuntimeError("rk3 step failed")
        return u

    def max_cfl(self, gamma, u, dt):
        return lib().orc_max_cfl(self.h, gamma, self._state(u), dt)

    def density_range(self, u):
        lo, hi = C.c_double(), C.c_double()
        lib().orc_density_range(self.h, self._state(u), C.byref(lo), C.byref(hi))
        return lo.value, hi.value

    def project(self, Uq):
        self._ensure_minv()
        Uq = np.ascontiguousarray(Uq, dtype=np.float64).reshape(self.ne, self.nq, 4)
        out = np.zeros((self.ne, self.np, 4))
        lib().orc_project(self.h, Uq, out)
        return out
