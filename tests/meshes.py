"""Test-side mesh and initial-condition helpers (numpy, independent of the product).

* ``two_triangle_mesh`` is dgfem's GMSH-free test mesh (tests/test_helpers.h:11-51),
  including its boundary-edge list, which names (element, face) pairs that dgfem then
  reads as vertex pairs.
* ``periodic_rectangle`` is an N x N quad grid split along each quad's (i,j)-(i+1,j+1)
  diagonal into two counter-clockwise triangles, with dgfem's GMSH physical tags
  Bottom=2, Right=3, Top=4, Left=5 (src/utils/mesh_creation.cpp:249-260).
* ``quad_rectangle`` is the same grid as counter-clockwise quadrilaterals, optionally
  with its interior vertices displaced (bilinear, non-affine elements).
"""

import numpy as np

BOTTOM, RIGHT, TOP, LEFT = 2, 3, 4, 5
TAGS = {"Bottom": BOTTOM, "Right": RIGHT, "Top": TOP, "Left": LEFT}
PERIODIC_PAIRS = ((LEFT, RIGHT, True), (BOTTOM, TOP, False))


def two_triangle_mesh():
    verts = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    elems = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int32)
    # {1: {(0,0)}, 2: {(0,1), (1,1)}, 3: {(1,2)}, 4: {(0,2)}} read as vertex pairs
    bedges = np.array([[1, 0, 0], [2, 0, 1], [2, 1, 1], [3, 1, 2], [4, 0, 2]], dtype=np.int32)
    return verts, elems, bedges


def periodic_rectangle(n, x0=-5.0, x1=5.0, y0=-5.0, y1=5.0, nx=None):
    nx = n if nx is None else nx
    ny = n
    xs = np.linspace(x0, x1, nx + 1)
    ys = np.linspace(y0, y1, ny + 1)
    X, Y = np.meshgrid(xs, ys)
    verts = np.stack([X.ravel(), Y.ravel()], axis=1)

    def vid(i, j):
        return j * (nx + 1) + i

    elems = []
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)
            elems.append((a, b, c))
            elems.append((a, c, d))
    be = []
    for i in range(nx):
        be.append((BOTTOM, vid(i, 0), vid(i + 1, 0)))
    for j in range(ny):
        be.append((RIGHT, vid(nx, j), vid(nx, j + 1)))
    for i in range(nx):
        be.append((TOP, vid(i, ny), vid(i + 1, ny)))
    for j in range(ny):
        be.append((LEFT, vid(0, j), vid(0, j + 1)))
    return verts, np.array(elems, dtype=np.int32), np.array(be, dtype=np.int32)


def primitive_to_conserved(W, gamma=1.4):
    W = np.asarray(W, dtype=np.float64)
    rho, u, v, p = W[..., 0], W[..., 1], W[..., 2], W[..., 3]
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.stack([rho, rho * u, rho * v, E], axis=-1)


def isentropic_vortex(xy, t=0.0, beta=5.0, xc=0.0, yc=0.0, uinf=0.5, vinf=0.0, gamma=1.4,
                      period=10.0):
    """Shu's isentropic vortex on the free stream rho=1, p=1, advected with (uinf, vinf)
    on a periodic box of side ``period`` (conserved variables)."""
    x = xy[..., 0] - (xc + uinf * t)
    y = xy[..., 1] - (yc + vinf * t)
    x = (x + period / 2) % period - period / 2
    y = (y + period / 2) % period - period / 2
    r2 = x * x + y * y
    g = beta / (2.0 * np.pi) * np.exp(0.5 * (1.0 - r2))
    u = uinf - y * g
    v = vinf + x * g
    T = 1.0 - (gamma - 1.0) / (2.0 * gamma) * g * g
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho * T
    return primitive_to_conserved(np.stack([rho, u, v, p], axis=-1), gamma)


def quad_rectangle(n, x0=-5.0, x1=5.0, y0=-5.0, y1=5.0, nx=None, distort=0.0, seed=0):
    nx = n if nx is None else nx
    ny = n
    xs = np.linspace(x0, x1, nx + 1)
    ys = np.linspace(y0, y1, ny + 1)
    X, Y = np.meshgrid(xs, ys)
    verts = np.stack([X.ravel(), Y.ravel()], axis=1)
    if distort:
        rng = np.random.default_rng(seed)
        hx, hy = (x1 - x0) / nx, (y1 - y0) / ny
        inner = (np.abs(verts[:, 0] - x0) > 1e-12) & (np.abs(verts[:, 0] - x1) > 1e-12) & \
                (np.abs(verts[:, 1] - y0) > 1e-12) & (np.abs(verts[:, 1] - y1) > 1e-12)
        verts = verts.copy()
        verts[inner] += distort * np.array([hx, hy]) * rng.uniform(-1, 1, (inner.sum(), 2))

    def vid(i, j):
        return j * (nx + 1) + i

    elems = [(vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)) for j in range(ny) for i in range(nx)]
    be = []
    for i in range(nx):
        be.append((BOTTOM, vid(i, 0), vid(i + 1, 0)))
    for j in range(ny):
        be.append((RIGHT, vid(nx, j), vid(nx, j + 1)))
    for i in range(nx):
        be.append((TOP, vid(i, ny), vid(i + 1, ny)))
    for j in range(ny):
        be.append((LEFT, vid(0, j), vid(0, j + 1)))
    return verts, np.array(elems, dtype=np.int32), np.array(be, dtype=np.int32)


def taylor_green(xy, seed=0, gamma=1.4, mach=0.1, noise=1e-3):
    """Decaying Taylor-Green-type vortex on [0, 2 pi]^2 (conserved variables): rho=1,
    u=sin x cos y, v=-cos x sin y, p = 1/(gamma M^2) + (cos 2x + cos 2y)/4, plus seeded
    Gaussian noise of amplitude ``noise`` on both velocity components."""
    x, y = xy[..., 0], xy[..., 1]
    rng = np.random.default_rng(seed)
    u = np.sin(x) * np.cos(y) + noise * rng.standard_normal(x.shape)
    v = -np.cos(x) * np.sin(y) + noise * rng.standard_normal(x.shape)
    p = 1.0 / (gamma * mach * mach) + 0.25 * (np.cos(2 * x) + np.cos(2 * y))
    rho = np.ones_like(x)
    return primitive_to_conserved(np.stack([rho, u, v, p], axis=-1), gamma)
