"""Python mirror of dgfem's public API for the explicit Euler / Navier-Stokes path.

Names, argument meanings and error behaviour follow dgfem (paths inside the dgfem
project); the work happens in libdgx.so on the GPU.

* ``DGMesh``            include/dgfem/core/mesh.hpp:29-228
* ``DGSpace``           include/dgfem/core/space.hpp:25-141 (order + basis choice)
* ``EulerWeakFormulation`` / ``NavierStokesWeakFormulation``
                        include/dgfem/weak_forms/{euler,navier_stokes}_weak_formulation.hpp
* ``DGAssembler``       include/dgfem/solver/assembler.hpp (assemble_euler_residual)
* ``EulerDGSolver`` / ``NavierStokesDGSolver``
                        include/dgfem/solver/dg_solver.hpp:223-296

States are ``(n_elements, n_basis, 4)`` float64 arrays: dgfem's per-element Np x 4
matrices.  numpy arrays run through the host entry points; CUDA torch tensors run on
the device on torch's current stream.
"""

from __future__ import annotations

import ctypes as C
from typing import Callable, Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib as L
from ._lib import check

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _stream_of(t):
    import torch
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


class BCTypeEuler:
    """include/dgfem/boundary/conditions.hpp:27-32"""
    FAR_FIELD = L.BC_FAR_FIELD
    SLIP_WALL = L.BC_SLIP_WALL
    NO_SLIP_WALL = L.BC_NO_SLIP_WALL
    PERIODIC = L.BC_PERIODIC


class BoundaryConditionEuler:
    """Constant-valued BoundaryConditionEuler (conditions.hpp:75-103)."""

    def __init__(self, bc_type: int, value: Sequence[float] = (0.0, 0.0, 0.0, 0.0)):
        self.type = int(bc_type)
        self.value = np.ascontiguousarray(value, dtype=np.float64).reshape(4)

    def get_type(self) -> int:
        return self.type

    def evaluate(self, x) -> np.ndarray:
        return self.value.copy()


def primitive_to_conserved(W, gamma: float = 1.4) -> np.ndarray:
    """euler_weak_formulation.cpp:261-277"""
    W = np.asarray(W, dtype=np.float64)
    rho, u, v, p = W[..., 0], W[..., 1], W[..., 2], W[..., 3]
    return np.stack([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)], -1)


def conserved_to_primitive(U, gamma: float = 1.4) -> np.ndarray:
    """euler_weak_formulation.cpp:279-296"""
    U = np.asarray(U, dtype=np.float64)
    rho = U[..., 0]
    ri = 1.0 / rho
    u, v = U[..., 1] * ri, U[..., 2] * ri
    return np.stack([rho, u, v, (gamma - 1.0) * (U[..., 3] - 0.5 * rho * (u * u + v * v))], -1)


class DGMesh:
    """DGMesh(vertices, elements, element_tags, boundary_tags, boundary_edges).

    ``boundary_edges`` maps a tag id to a list of (v1, v2) vertex pairs, as in dgfem."""

    def __init__(self, vertices, elements, element_tags=None,
                 boundary_tags: Optional[Dict[str, int]] = None,
                 boundary_edges: Optional[Dict[int, Iterable[Tuple[int, int]]]] = None,
                 _handle=None):
        lib = L.load()
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            V = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 2)
            E = np.asarray(elements)
            nvpe = E.shape[1] if E.ndim == 2 else 3  # 3: triangles, 4: quadrilaterals (mesh.cpp:23-35)
            E = np.ascontiguousarray(E, dtype=np.int32).reshape(-1, nvpe)
            tags = boundary_tags or {}
            names = (C.c_char_p * max(1, len(tags)))(*[k.encode() for k in tags])
            ids = np.ascontiguousarray(list(tags.values()) or [0], dtype=np.int32)
            be = []
            for tag in sorted((boundary_edges or {}).keys()):
                for v1, v2 in boundary_edges[tag]:
                    be.append((tag, v1, v2))
            B = np.ascontiguousarray(be if be else np.zeros((0, 3)), dtype=np.int32).reshape(-1, 3)
            check(lib.dgx_mesh_create_nv(nvpe, len(V), _dptr(V), len(E), _iptr(E), len(tags), names,
                                         _iptr(ids), len(B), _iptr(B), C.byref(self._h)))
        self._bc_keep = []

    @classmethod
    def rectangle(cls, nx: int, ny: int, x0: float, x1: float, y0: float, y1: float,
                  periodic: bool = True, element_type: str = "triangle") -> "DGMesh":
        """Structured mesh of a rectangle, two triangles per cell or ``element_type="quad"``
        cells (tags Bottom=2 Right=3 Top=4 Left=5)."""
        h = C.c_void_p()
        if element_type not in ("triangle", "quad"):
            raise ValueError(f"Unknown element type: {element_type}")
        fn = L.load().dgx_mesh_create_rectangle_quad if element_type == "quad" else L.load().dgx_mesh_create_rectangle
        check(fn(nx, ny, x0, x1, y0, y1, int(periodic), C.byref(h)))
        return cls(None, None, _handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.load().dgx_mesh_destroy(h)
            self._h = None

    def set_periodic_boundaries(self, tag1: str, tag2: str):
        check(L.load().dgx_mesh_set_periodic(self._h, tag1.encode(), tag2.encode()))

    def set_boundary_condition_euler(self, tag: str, bc: BoundaryConditionEuler):
        check(L.load().dgx_mesh_set_bc(self._h, tag.encode(), bc.type, _dptr(bc.value)))
        self._bc_keep.append(bc)

    def _info(self):
        ne, nif, nbf = C.c_int(), C.c_int(), C.c_int()
        check(L.load().dgx_mesh_info(self._h, C.byref(ne), C.byref(nif), C.byref(nbf)))
        return ne.value, nif.value, nbf.value

    def get_n_elements(self) -> int:
        return self._info()[0]

    def get_interior_faces(self) -> np.ndarray:
        """(n, 5): elem_L, elem_R, face_L, face_R, reversed."""
        n = self._info()[1]
        out = np.zeros((n, 5), np.int32)
        if n:
            check(L.load().dgx_mesh_interior_faces(self._h, _iptr(out)))
        return out

    def get_boundary_face_data(self) -> np.ndarray:
        """(n, 3): elem, face, tag id."""
        n = self._info()[2]
        out = np.zeros((n, 3), np.int32)
        if n:
            check(L.load().dgx_mesh_boundary_faces(self._h, _iptr(out)))
        return out

    def get_vertices(self) -> np.ndarray:
        nv = C.c_int()
        check(L.load().dgx_mesh_arrays(self._h, C.byref(nv), None, None))
        V = np.zeros((nv.value, 2))
        check(L.load().dgx_mesh_arrays(self._h, None, _dptr(V), None))
        return V

    def get_element_type(self) -> str:
        """"triangle" or "quad" (DGMesh::get_element_type)."""
        return "quad" if self.vertices_per_element() == 4 else "triangle"

    def vertices_per_element(self) -> int:
        n = C.c_int()
        check(L.load().dgx_mesh_vertices_per_element(self._h, C.byref(n)))
        return n.value

    def get_elements(self) -> np.ndarray:
        E = np.zeros((self.get_n_elements(), self.vertices_per_element()), np.int32)
        check(L.load().dgx_mesh_arrays(self._h, None, None, _iptr(E)))
        return E


class DGSpace:
    """DGSpace("triangle", order) with a basis choice (dgfem's default is monomial), or
    DGSpace("quad", order), whose basis is LegendreBasis (space.cpp:307-319)."""

    def __init__(self, element_type: str = "triangle", order: int = 1, basis: Optional[str] = None):
        if element_type not in ("triangle", "quad"):
            raise ValueError(f"Unknown element type: {element_type}")
        if order < 1 or order > 10:
            raise ValueError(f"Element order must be between 1 and 10, got: {order}")
        self.element_type = element_type
        self.order = order
        if basis is None:
            basis = "legendre" if element_type == "quad" else "monomial"
        if (basis == "legendre") != (element_type == "quad"):
            raise ValueError(f"basis {basis!r} does not apply to {element_type} elements")
        self.basis = {"monomial": L.BASIS_MONOMIAL, "dubiner": L.BASIS_DUBINER,
                      "legendre": L.BASIS_LEGENDRE}[basis]

    def get_order(self) -> int:
        return self.order


class EulerWeakFormulation:
    def __init__(self, gamma: float = 1.4):
        self.gamma = gamma

    def get_gamma(self) -> float:
        return self.gamma

    def has_viscous_terms(self) -> bool:
        return False

    def get_n_vars(self) -> int:
        return 4


class NavierStokesWeakFormulation(EulerWeakFormulation):
    def __init__(self, gamma=1.4, dynamic_viscosity=1.0e-3, prandtl=0.72, penalty_prefactor=5.0):
        super().__init__(gamma)
        if dynamic_viscosity <= 0.0:
            raise ValueError("Dynamic viscosity must be positive for Navier-Stokes weak formulation")
        if prandtl <= 0.0:
            raise ValueError("Prandtl number must be positive for Navier-Stokes weak formulation")
        if penalty_prefactor <= 0.0:
            raise ValueError("Penalty prefactor must be positive for Navier-Stokes weak formulation")
        self.mu = dynamic_viscosity
        self.prandtl = prandtl
        self.sigma0 = penalty_prefactor

    def has_viscous_terms(self) -> bool:
        return True

    def compute_penalty_parameter(self, p: int, h: float) -> float:
        return self.sigma0 * self.mu * (p + 1) * (p + 1) / max(h, 1e-12)


class DGContext:
    """The device-resident solver behind DGAssembler / the solvers (one dgx_ctx)."""

    def __init__(self, mesh: DGMesh, space: DGSpace, weak_form: EulerWeakFormulation,
                 precision: str = "fp64"):
        lib = L.load()
        visc = weak_form.has_viscous_terms()
        p = L.Params(space.order, space.basis, L.NAVIER_STOKES if visc else L.EULER,
                     {"fp64": L.FP64, "mixed": L.MIXED, "df64": L.DF64}[precision], weak_form.gamma,
                     getattr(weak_form, "mu", 0.0), getattr(weak_form, "prandtl", 0.0),
                     getattr(weak_form, "sigma0", 0.0))
        self._h = C.c_void_p()
        check(lib.dgx_create(mesh._h, C.byref(p), C.byref(self._h)))
        ne, nb, nq, nfq = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib.dgx_info(self._h, C.byref(ne), C.byref(nb), C.byref(nq), C.byref(nfq)))
        self.n_elements, self.n_basis, self.n_quad, self.n_face_quad = ne.value, nb.value, nq.value, nfq.value
        self.shape = (self.n_elements, self.n_basis, 4)
        self.mesh, self.space, self.weak_form, self.precision = mesh, space, weak_form, precision

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.load().dgx_destroy(h)
            self._h = None

    # ---- helpers
    def _host(self, a) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != int(np.prod(self.shape)):
            raise ValueError(f"state has {a.size} values, expected {self.shape}")
        return a.reshape(self.shape)

    def _dev(self, t):
        import torch
        if t.dtype != torch.float64 or not t.is_cuda or not t.is_contiguous():
            raise ValueError("device states must be contiguous float64 CUDA tensors")
        if t.numel() != int(np.prod(self.shape)):
            raise ValueError(f"state has {t.numel()} values, expected {self.shape}")
        return C.c_void_p(t.data_ptr())

    # ---- hot path
    def residual(self, u, out=None):
        lib = L.load()
        if _is_torch(u):
            import torch
            out = torch.empty_like(u) if out is None else out
            check(lib.dgx_residual(self._h, self._dev(u), self._dev(out), _stream_of(u)))
            return out
        u = self._host(u)
        out = np.empty(self.shape) if out is None else out
        check(lib.dgx_residual_host(self._h, _dptr(u), _dptr(out)))
        return out

    def rhs(self, u, out=None):
        import torch
        lib = L.load()
        out = torch.empty_like(u) if out is None else out
        check(lib.dgx_rhs(self._h, self._dev(u), self._dev(out), _stream_of(u)))
        return out

    def apply_mass_inv(self, r, out=None):
        import torch
        out = torch.empty_like(r) if out is None else out
        check(L.load().dgx_apply_mass_inv(self._h, self._dev(r), self._dev(out), _stream_of(r)))
        return out

    def rk3_step(self, u, dt: float, n_steps: int = 1):
        """In place for CUDA tensors; returns a new array for numpy input."""
        lib = L.load()
        if _is_torch(u):
            check(lib.dgx_rk3_step(self._h, self._dev(u), float(dt), int(n_steps), _stream_of(u)))
            return u
        u = np.array(self._host(u), copy=True)
        check(lib.dgx_rk3_step_host(self._h, _dptr(u), float(dt), int(n_steps)))
        return u

    def rk3_stage(self, u_n, u_s, out, dt: float, stage: int):
        """One SSP-RK3 stage on CUDA tensors (dgx_rk3_stage; FP64 and df64 contexts): the stage
        the step makes, for drivers that exchange data between stages (dgfem_gb300.partition)."""
        check(L.load().dgx_rk3_stage(self._h, self._dev(u_n), self._dev(u_s), self._dev(out), float(dt), int(stage),
                                     _stream_of(out)))
        return out

    def launch_shape(self) -> Tuple[int, int, bool]:
        """(grid, tiles, tensor_cores) of the mixed stage kernel; grid is 0 until the first
        rk3_step; tensor_cores is True for the 3xTF32 tcgen05 form."""
        g, t, k = C.c_int(), C.c_int(), C.c_int()
        check(L.load().dgx_launch_shape(self._h, C.byref(g), C.byref(t), C.byref(k)))
        return g.value, t.value, k.value == 1

    def stage_tile(self) -> int:
        """Elements per CTA of the mixed stage kernel (128, or 64 / 32 for the face-trace form at
        smaller tiles); 0 until the first rk3_step."""
        k = C.c_int()
        check(L.load().dgx_stage_tile(self._h, C.byref(k), None))
        return k.value

    def stage_nbr_shared(self) -> bool:
        """True when the mixed stage kernel copies each element's neighbour trace blocks into
        shared memory during staging (the face-trace form at 32-element tiles)."""
        k, n = C.c_int(), C.c_int()
        check(L.load().dgx_stage_tile(self._h, C.byref(k), C.byref(n)))
        return n.value == 1

    def stage_form(self) -> str:
        """The mixed stage kernel's form: "rows" (neighbour coefficient rows per face),
        "traces" (face traces through HBM), "traces pipelined" (the same, each CTA copying its
        next tile's inputs while it computes one) or "tensor cores"."""
        k = C.c_int()
        check(L.load().dgx_launch_shape(self._h, None, None, C.byref(k)))
        return {0: "rows", 1: "tensor cores", 2: "traces", 3: "traces pipelined"}[k.value]

    def quad_points(self) -> np.ndarray:
        xq = np.zeros((self.n_elements, self.n_quad, 2))
        check(L.load().dgx_quad_points(self._h, _dptr(xq)))
        return xq

    def quad_points_device(self):
        """quad_points() as a CUDA tensor, for evaluating an initial condition on the GPU."""
        import torch
        xq = torch.empty((self.n_elements, self.n_quad, 2), dtype=torch.float64, device="cuda")
        check(L.load().dgx_quad_points_device(self._h, C.c_void_p(xq.data_ptr()),
                                              C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return xq

    def project(self, uq):
        """L2 projection of values at quad_points() (device tensor in, device tensor out)."""
        import torch
        out = torch.empty(self.shape, dtype=torch.float64, device=uq.device)
        check(L.load().dgx_project(self._h, C.c_void_p(uq.data_ptr()), self._dev(out), _stream_of(uq)))
        return out

    def max_cfl(self, u, dt: float) -> float:
        r = C.c_double()
        check(L.load().dgx_max_cfl(self._h, self._dev(u), float(dt), C.byref(r), _stream_of(u)))
        return r.value

    def density_range(self, u) -> Tuple[float, float]:
        lo, hi = C.c_double(), C.c_double()
        check(L.load().dgx_density_range(self._h, self._dev(u), C.byref(lo), C.byref(hi), _stream_of(u)))
        return lo.value, hi.value

    def step_nonfinite(self) -> bool:
        """True when an RK3 step since the last call produced a NaN or Inf (device flag, read
        and cleared on torch's current stream).  Raises DGXError (DGX_ERR_TIMEOUT) when a
        bounded wait inside the tensor-core stage kernel gave up."""
        import torch
        f = C.c_int()
        rc = L.load().dgx_step_status(self._h, C.byref(f), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc not in (L.OK, L.ERR_NONFINITE):
            check(rc)
        return bool(f.value)

    def has_nan(self, u) -> bool:
        f = C.c_int()
        check(L.load().dgx_has_nan(self._h, self._dev(u), C.byref(f), _stream_of(u)))
        return bool(f.value)

    # ---- differentiation (FP64 contexts)
    def residual_jvp(self, u, du):
        """(dR/du) du, the tangent of assemble_euler_residual."""
        import torch
        out = torch.empty_like(u)
        check(L.load().dgx_residual_jvp(self._h, self._dev(u), self._dev(du), self._dev(out), _stream_of(u)))
        return out

    def residual_vjp(self, u, rbar):
        """(dR/du)^T rbar (Euler)."""
        import torch
        out = torch.empty_like(u)
        check(L.load().dgx_residual_vjp(self._h, self._dev(u), self._dev(rbar), self._dev(out), _stream_of(u)))
        return out

    def rk3_step_tlm(self, u, du, dt: float, n_steps: int = 1):
        """Advance (u, du) in place through n_steps tangent-linear SSP-RK3 steps."""
        check(L.load().dgx_rk3_step_tlm(self._h, self._dev(u), self._dev(du), float(dt), int(n_steps),
                                        _stream_of(u)))
        return u, du

    def rk3_step_adjoint(self, u_n, ubar, dt: float):
        """Replace ubar (cotangent of u^{n+1}) by the cotangent of u_n, in place."""
        check(L.load().dgx_rk3_step_adjoint(self._h, self._dev(u_n), self._dev(ubar), float(dt), _stream_of(u_n)))
        return ubar

    def kinetic_energy(self, u, grad: bool = False):
        """J = integral of rho |u|^2 / 2 at the volume points (and dJ/du when grad)."""
        import torch
        J = C.c_double()
        g = torch.empty_like(u) if grad else None
        check(L.load().dgx_kinetic_energy(self._h, self._dev(u), C.byref(J),
                                          self._dev(g) if grad else None, _stream_of(u)))
        return (J.value, g) if grad else J.value

    def kinetic_energy_gradient(self, u0, dt: float, n_steps: int, checkpoint_every: int = 50):
        """(J(u(T)), dJ/du0) by the checkpointed adjoint."""
        import torch
        J = C.c_double()
        g = torch.empty_like(u0)
        check(L.load().dgx_kinetic_energy_gradient(self._h, self._dev(u0), float(dt), int(n_steps),
                                                   int(checkpoint_every), C.byref(J), self._dev(g),
                                                   _stream_of(u0)))
        return J.value, g

    def kinetic_energy_gradient_binomial(self, u0, dt: float, n_steps: int, n_snapshots: int):
        """(J(u(T)), dJ/du0, stats) by binomial checkpointing with n_snapshots device states;
        stats = {"recomputed_steps", "states_held", "optimal_recomputed_steps"}."""
        import torch
        J = C.c_double()
        g = torch.empty_like(u0)
        st = (C.c_longlong * 3)()
        check(L.load().dgx_kinetic_energy_gradient_binomial(self._h, self._dev(u0), float(dt), int(n_steps),
                                                            int(n_snapshots), C.byref(J), self._dev(g), st,
                                                            _stream_of(u0)))
        return J.value, g, {"recomputed_steps": int(st[0]), "states_held": int(st[1]),
                            "optimal_recomputed_steps": int(st[2])}


class _DeviceArray:
    """CUDA array interface over float64 device memory owned by a DGBatch (torch.as_tensor
    wraps it without a copy; the tensor keeps this object, and so the batch, alive)."""

    def __init__(self, owner, ptr: int, shape):
        self._owner = owner
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 2, "strides": None}


class DGBatch:
    """Independent mixed-precision Euler or Navier-Stokes solves advanced together
    (include/dgx.h dgx_batch_*).

    ``meshes[i]`` and ``spaces[i]`` (order 1..4, one basis for all) define instance i; the
    weak form (its physics and parameters) is shared; every RK3 stage of every instance is
    one persistent kernel launch.  ``state(i)`` is a CUDA
    float64 tensor view of instance i's state, shape (n_elements, n_basis, 4), owned by the
    batch.  No counterpart in dgfem, where an ensemble is a loop over solver objects."""

    def __init__(self, meshes: Sequence[DGMesh], spaces: Sequence[DGSpace],
                 weak_form: Optional[EulerWeakFormulation] = None):
        if len(meshes) != len(spaces) or not meshes:
            raise ValueError("DGBatch needs one space per mesh and at least one instance")
        wf = weak_form or EulerWeakFormulation()
        visc = wf.has_viscous_terms()
        phys = (L.NAVIER_STOKES, wf.mu, wf.prandtl, wf.sigma0) if visc else (L.EULER, 0.0, 0.0, 0.0)
        lib = L.load()
        n = len(meshes)
        prm = (L.Params * n)(*[L.Params(s.order, s.basis, phys[0], L.MIXED, wf.gamma, *phys[1:]) for s in spaces])
        hs = (C.c_void_p * n)(*[m._h.value for m in meshes])
        self._h = C.c_void_p()
        check(lib.dgx_batch_create(n, hs, C.cast(prm, C.c_void_p), C.byref(self._h)))
        self.n_instances = n
        self.meshes, self.spaces, self.weak_form = list(meshes), list(spaces), wf
        self.shapes = []
        self._ptrs = []
        for i in range(n):
            ne, nb, ptr = C.c_int(), C.c_int(), C.c_void_p()
            check(lib.dgx_batch_info(self._h, i, C.byref(ne), C.byref(nb), C.byref(ptr)))
            self.shapes.append((ne.value, nb.value, 4))
            self._ptrs.append(ptr.value)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.load().dgx_batch_destroy(h)
            self._h = None

    def state(self, i: int):
        """Instance i's FP64 state as a CUDA tensor view (write initial states into it)."""
        import torch
        if not 0 <= i < self.n_instances:
            raise IndexError("instance index out of range")
        return torch.as_tensor(_DeviceArray(self, self._ptrs[i], self.shapes[i]), device="cuda")

    def rk3_step(self, dt, n_steps: int = 1):
        """n_steps SSP-RK3 steps of every instance on torch's current stream; dt is one step
        for all instances or a sequence with one per instance."""
        import torch
        d = np.broadcast_to(np.asarray(dt, dtype=np.float64), (self.n_instances,)).copy()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        check(L.load().dgx_batch_rk3_step(self._h, _dptr(d), int(n_steps), stream))

    def launch_shape(self) -> Tuple[int, int]:
        """(grid, tiles) of the batched stage kernel; grid is 0 until the first step."""
        g, t = C.c_int(), C.c_int()
        check(L.load().dgx_batch_launch_shape(self._h, C.byref(g), C.byref(t)))
        return g.value, t.value

    def stage_form(self) -> str:
        """The batch's stage form: "batched rows" (one launch per stage over every order's tiles)
        or "traces per order" (the face-trace kernel, one launch per order); "" until the first
        rk3_step."""
        k = C.c_int()
        check(L.load().dgx_batch_stage_form(self._h, C.byref(k)))
        return {0: "", 1: "batched rows", 2: "traces per order"}[k.value]


class DGAssembler:
    """DGAssembler(mesh, weak_form) with assemble_euler_residual (assembler.hpp:58-59)."""

    def __init__(self, mesh: DGMesh, weak_form: EulerWeakFormulation, space: DGSpace,
                 precision: str = "fp64"):
        self.ctx = DGContext(mesh, space, weak_form, precision)

    def assemble_euler_residual(self, u_coeffs, residuals_out=None):
        return self.ctx.residual(u_coeffs, residuals_out)


class CompressibleDGSolverBase:
    """include/dgfem/solver/dg_solver.hpp:223-257 on the GPU."""

    def __init__(self, mesh: DGMesh, weak_form: EulerWeakFormulation, space: DGSpace,
                 precision: str = "fp64", device: str = "cuda"):
        self.ctx = DGContext(mesh, space, weak_form, precision)
        self.weak_form = weak_form
        self.device = device
        self.verbose = False
        self.telemetry = {"steps_completed": 0, "rhs_evaluations": 0, "output_frames": 0}

    def project_initial_condition(self, u0_func: Callable[[np.ndarray], np.ndarray]):
        """u0_func maps (..., 2) physical points to (..., 4) conserved states."""
        import torch
        xq = self.ctx.quad_points()
        uq = torch.as_tensor(np.ascontiguousarray(u0_func(xq), dtype=np.float64), device=self.device)
        return self.ctx.project(uq)

    def assemble_residual(self, u):
        self.telemetry["rhs_evaluations"] += 1
        return self.ctx.residual(u)

    def apply_mass_inv(self, r):
        return self.ctx.apply_mass_inv(r)

    def time_step_ssp_rk3(self, u_n, dt: float):
        u = u_n.clone() if _is_torch(u_n) else u_n
        self.telemetry["rhs_evaluations"] += 3
        return self.ctx.rk3_step(u, dt, 1)

    def compute_max_cfl(self, u, dt: float) -> float:
        return self.ctx.max_cfl(u, dt)

    def compute_density_range(self, u) -> Tuple[float, float]:
        return self.ctx.density_range(u)

    def solve(self, initial_condition, T_final: float, dt: float, save_every: int = 1) -> List[np.ndarray]:
        """run_time_integration (compressible_solver_base.cpp:201-338): frames flattened to
        (n_elements, n_basis*4) every save_every steps; NaN aborts the loop."""
        u = self.project_initial_condition(initial_condition)
        frames = [u.clone()]
        t, step = 0.0, 0
        while t < T_final:
            if step % save_every == 0 and step > 0:
                frames.append(u.clone())
            self.ctx.rk3_step(u, dt, 1)
            t += dt
            step += 1
            self.telemetry["steps_completed"] += 1
            self.telemetry["rhs_evaluations"] += 3
            if self.ctx.step_nonfinite():  # dgfem's per-step NaN check: stop the run
                break
        if step % save_every != 0:
            frames.append(u.clone())
        self.telemetry["output_frames"] += len(frames)
        ne, nb = self.ctx.n_elements, self.ctx.n_basis
        return [f.reshape(ne, nb * 4).cpu().numpy() for f in frames]


class EulerDGSolver(CompressibleDGSolverBase):
    def __init__(self, mesh: DGMesh, space: DGSpace, gamma: float = 1.4, precision: str = "fp64"):
        super().__init__(mesh, EulerWeakFormulation(gamma), space, precision)


class NavierStokesDGSolver(CompressibleDGSolverBase):
    def __init__(self, mesh: DGMesh, space: DGSpace, gamma=1.4, dynamic_viscosity=1.0e-3,
                 prandtl=0.72, penalty_prefactor=5.0, precision: str = "fp64"):
        super().__init__(mesh, NavierStokesWeakFormulation(gamma, dynamic_viscosity, prandtl,
                                                            penalty_prefactor), space, precision)


def _autograd():
    import torch

    class RK3Trajectory(torch.autograd.Function):
        """u(T) = n_steps SSP-RK3 steps from u0; the backward pass is the hand-written adjoint
        with a checkpoint every `checkpoint_every` steps and recomputation in between."""

        @staticmethod
        def forward(fctx, u0, dgctx, dt, n_steps, checkpoint_every):
            u = u0.detach().clone()
            cks = [u.clone()]
            for n in range(n_steps):
                dgctx.rk3_step(u, dt, 1)
                if (n + 1) % checkpoint_every == 0 and n + 1 < n_steps:
                    cks.append(u.clone())
            fctx.dgctx, fctx.dt, fctx.n, fctx.ce, fctx.cks = dgctx, dt, n_steps, checkpoint_every, cks
            return u

        @staticmethod
        def backward(fctx, gT):
            dg, dt, n, ce = fctx.dgctx, fctx.dt, fctx.n, fctx.ce
            ubar = gT.detach().clone().contiguous()
            nseg = len(fctx.cks)
            for g in range(nseg - 1, -1, -1):
                n0, n1 = g * ce, min(n, (g + 1) * ce)
                states = [fctx.cks[g].clone()]
                for _ in range(n0, n1 - 1):
                    u = states[-1].clone()
                    dg.rk3_step(u, dt, 1)
                    states.append(u)
                for k in range(n1 - n0 - 1, -1, -1):
                    dg.rk3_step_adjoint(states[k], ubar, dt)
            return ubar, None, None, None, None

    class KineticEnergy(torch.autograd.Function):
        """J = integral of rho |u|^2 / 2 over the domain at the volume quadrature points."""

        @staticmethod
        def forward(fctx, u, dgctx):
            J, g = dgctx.kinetic_energy(u.detach().contiguous(), grad=True)
            fctx.save_for_backward(g)
            return torch.tensor(J, dtype=torch.float64, device=u.device)

        @staticmethod
        def backward(fctx, gJ):
            (g,) = fctx.saved_tensors
            return gJ * g, None

    return RK3Trajectory, KineticEnergy


def rk3_trajectory(u0, dgctx: DGContext, dt: float, n_steps: int, checkpoint_every: int = 50):
    """Differentiable SSP-RK3 trajectory (torch.autograd), FP64 Euler contexts."""
    return _autograd()[0].apply(u0, dgctx, dt, n_steps, checkpoint_every)


def kinetic_energy(u, dgctx: DGContext):
    """Differentiable kinetic-energy objective (torch.autograd)."""
    return _autograd()[1].apply(u, dgctx)
