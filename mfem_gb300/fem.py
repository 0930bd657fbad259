"""Host-side discretisation data for the PA path: 1D quadrature and basis
tables, structured hexahedral meshes, the H1 dof numbering, and the seeded
synthetic inputs (jittered vertices, lognormal coefficient). Everything here is
set-up work done once per problem; the hot path is the CUDA library.

Conventions follow MFEM's:
  * Gauss-Legendre rules on [0, 1] (fem/intrules.cpp:620-690); the 3D tensor
    weight is W[ix + Q*(iy + Q*iz)] = w[ix] w[iy] w[iz].
  * H1 basis = Lagrange polynomials on the Gauss-Lobatto points
    (fem/fe_coll.hpp:300-302, fem/fe/fe_base.cpp:2697-2741); tables are
    column-major (Q, D): B[q + Q*d] = phi_d(x_q).
  * Element dofs in lexicographic order (the LEXICOGRAPHIC ElementRestriction
    ordering, fem/restriction.cpp:40-66).
"""
import math

import numpy as np

MASK64 = (1 << 64) - 1


# ------------------------------------------------------------ quadrature / basis
def gauss_legendre(n):
    """n-point Gauss-Legendre points and weights on [0, 1]."""
    x, w = np.polynomial.legendre.leggauss(n)
    # Newton polish on P_n for full double accuracy of the mapped points
    for _ in range(2):
        p0, p1 = np.ones_like(x), x.copy()
        for j in range(2, n + 1):
            p0, p1 = p1, ((2 * j - 1) * x * p1 - (j - 1) * p0) / j
        dp = n * (x * p1 - p0) / (x * x - 1) if n > 1 else np.ones_like(x)
        x = x - p1 / dp
    p0, p1 = np.ones_like(x), x.copy()
    for j in range(2, n + 1):
        p0, p1 = p1, ((2 * j - 1) * x * p1 - (j - 1) * p0) / j
    dp = n * (x * p1 - p0) / (x * x - 1) if n > 1 else np.ones_like(x)
    w = 2.0 / ((1 - x * x) * dp * dp) if n > 1 else np.array([2.0])
    xs = (x + 1) / 2
    order = np.argsort(xs)
    return xs[order], (w / 2)[order]


def gauss_lobatto(n):
    """n Gauss-Lobatto points on [0, 1] (endpoints plus zeros of P'_{n-1})."""
    if n == 1:
        return np.array([0.5])
    N = n - 1
    inner = np.polynomial.legendre.Legendre.basis(N).deriv().roots().real if N > 1 else np.array([])
    z = np.sort(inner)
    for _ in range(3):   # Newton polish on P'_N
        p0, p1 = np.ones_like(z), z.copy()
        for j in range(2, N + 1):
            p0, p1 = p1, ((2 * j - 1) * z * p1 - (j - 1) * p0) / j
        dp = N * (z * p1 - p0) / (z * z - 1)
        d2p = (2 * z * dp - N * (N + 1) * p1) / (1 - z * z)
        z = z - dp / d2p
    pts = np.concatenate([[-1.0], z, [1.0]])
    x = (pts + 1) / 2
    x = 0.5 * (x + (1 - x[::-1]))   # exact symmetry
    x[0], x[-1] = 0.0, 1.0
    return x


def basis_tables(nodes, xq):
    """Lagrange basis on `nodes` and its derivative at `xq`: (B, G), each
    column-major (Q, D) flattened."""
    D, Q = len(nodes), len(xq)
    B = np.zeros((D, Q))
    G = np.zeros((D, Q))
    for j in range(D):
        others = [m for m in range(D) if m != j]
        den = np.prod([nodes[j] - nodes[m] for m in others]) if others else 1.0
        for qi, y in enumerate(xq):
            B[j, qi] = np.prod([y - nodes[m] for m in others]) / den if others else 1.0
            s = 0.0
            for k in others:
                s += np.prod([y - nodes[m] for m in others if m != k])
            G[j, qi] = s / den
    return B.reshape(-1), G.reshape(-1)   # (D, Q) C-order == (Q, D) column-major


def tensor_weights(w):
    return np.einsum("k,j,i->kji", w, w, w).reshape(-1)


class Tables:
    """1D tables of an H1 order-p space at a Q-point Gauss-Legendre rule."""

    def __init__(self, p, q):
        self.p, self.D, self.Q = p, p + 1, q
        self.xq, self.wq = gauss_legendre(q)
        self.nodes = gauss_lobatto(p + 1)
        self.B, self.G = basis_tables(self.nodes, self.xq)
        self.W = tensor_weights(self.wq)


# ------------------------------------------------------------ synthetic inputs
def splitmix64(state):
    """Returns (value, new_state); the same stream the golden driver uses."""
    state = (state + 0x9E3779B97F4A7C15) & MASK64
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31), state


def u01_stream(seed, count):
    out = np.empty(count)
    s = seed
    for i in range(count):
        v, s = splitmix64(s)
        out[i] = (v >> 11) * (1.0 / 9007199254740992.0)
    return out


def u01_array(seed, count):
    """Vectorised splitmix64 stream (same values as u01_stream)."""
    idx = np.arange(1, count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def kappa_modes(seed=3):
    """16 Fourier modes k in Z^3 (|k|_inf <= 4), phases in [0, 2pi)."""
    u = u01_stream(seed, 64)
    k = np.zeros((16, 3), np.int64)
    phi = np.zeros(16)
    for i in range(16):
        for d in range(3):
            k[i, d] = int(u[4 * i + d] * 9.0) - 4
        phi[i] = 2.0 * math.pi * u[4 * i + 3]
    return k, phi


def kappa_eval(xyz, modes):
    """kappa(x) = exp(sum_m 0.5 cos(2 pi k_m . x + phi_m)); xyz (..., 3)."""
    k, phi = modes
    g = 0.0
    for m in range(16):
        a = 2.0 * math.pi * (k[m, 0] * xyz[..., 0] + k[m, 1] * xyz[..., 1] + k[m, 2] * xyz[..., 2]) + phi[m]
        g = g + 0.5 * np.cos(a) if isinstance(xyz, np.ndarray) else g + 0.5 * a.cos()
    return np.exp(g) if isinstance(xyz, np.ndarray) else g.exp()


# ------------------------------------------------------------------ meshes
class CartesianMesh:
    """n x n x n hexahedra of the unit cube. Vertices are numbered x fastest
    (as Mesh::MakeCartesian3D does); interior vertices may be jittered by
    U(-amp h, amp h) per coordinate from the splitmix64 stream (three draws per
    vertex, vertex order). Elements are numbered lexicographically."""

    def __init__(self, n, jitter=0.0, seed=1, curved=False):
        self.n = n
        self.ne = n ** 3
        self.nv = (n + 1) ** 3
        g = np.arange(n + 1) / n
        vz, vy, vx = np.meshgrid(g, g, g, indexing="ij")
        v = np.stack([vx.ravel(), vy.ravel(), vz.ravel()], axis=1).copy()
        if jitter > 0:
            h = 1.0 / n
            u = u01_array(seed, 3 * self.nv).reshape(self.nv, 3)
            interior = np.all((v > 1e-12) & (v < 1.0 - 1e-12), axis=1)
            v[interior] += (2.0 * u[interior] - 1.0) * jitter * h
        self.vertices = v
        self.curved = curved
        # element attributes (1-based, as Mesh::GetAttribute): all 1, as
        # MakeCartesian3D sets them; a caller may assign its own
        self.attributes = np.ones(self.ne, np.int32)

    def element_corners(self):
        """(NE, 8) vertex ids in lexicographic corner order (ax fastest)."""
        n = self.n
        ez, ey, ex = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        ex, ey, ez = ex.ravel(), ey.ravel(), ez.ravel()
        out = np.empty((self.ne, 8), np.int64)
        for az in range(2):
            for ay in range(2):
                for ax in range(2):
                    out[:, ax + 2 * (ay + 2 * az)] = (ex + ax) + (n + 1) * ((ey + ay) + (n + 1) * (ez + az))
        return out

    def nodes_evector(self, order=1):
        """Lexicographic nodes E-vector (Dg, Dg, Dg, 3, NE) flattened, for an
        order-`order` H1 geometry (order 1: the vertices; order > 1: the
        trilinear map sampled at Gauss-Lobatto points, then the curved map
        x + 0.05 sin(2 pi x) sin(2 pi y) sin(2 pi z) if `curved`)."""
        corners = self.vertices[self.element_corners()]          # (NE, 8, 3)
        if order == 1 and not self.curved:
            return np.ascontiguousarray(corners.transpose(0, 2, 1)).reshape(-1)
        pts = gauss_lobatto(order + 1)
        Dg = order + 1
        xi = np.stack(np.meshgrid(pts, pts, pts, indexing="ij")[::-1], axis=-1).reshape(-1, 3)
        # trilinear shape functions at xi, corner index ax + 2(ay + 2az)
        N = np.empty((Dg ** 3, 8))
        for az in range(2):
            for ay in range(2):
                for ax in range(2):
                    fx = xi[:, 0] if ax else 1 - xi[:, 0]
                    fy = xi[:, 1] if ay else 1 - xi[:, 1]
                    fz = xi[:, 2] if az else 1 - xi[:, 2]
                    N[:, ax + 2 * (ay + 2 * az)] = fx * fy * fz
        X = np.einsum("pa,eac->epc", N, corners)                   # (NE, Dg^3, 3)
        if self.curved:
            s = 0.05 * np.sin(2 * np.pi * X[..., 0]) * np.sin(2 * np.pi * X[..., 1]) * np.sin(2 * np.pi * X[..., 2])
            X = X + s[..., None]
        return np.ascontiguousarray(X.transpose(0, 2, 1)).reshape(-1)


class H1Space:
    """Order-p H1 space on a CartesianMesh with a global lexicographic dof
    grid ((p n + 1)^3 dofs). The element-to-dof table is already in
    lexicographic element order, so the restriction's dof_map is the identity."""

    def __init__(self, mesh, p):
        self.mesh, self.p, self.D = mesh, p, p + 1
        n = mesh.n
        self.N1 = p * n + 1
        self.ndofs = self.N1 ** 3
        self.ne = mesh.ne

    def element_dofs(self):
        n, p, D, N1 = self.mesh.n, self.p, self.D, self.N1
        ez, ey, ex = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        base = (p * ex.ravel()) + N1 * ((p * ey.ravel()) + N1 * (p * ez.ravel()))
        dz, dy, dx = np.meshgrid(np.arange(D), np.arange(D), np.arange(D), indexing="ij")
        loc = (dx.ravel() + N1 * (dy.ravel() + N1 * dz.ravel()))
        return (base[:, None] + loc[None, :]).astype(np.int32).reshape(-1)

    def boundary_dofs(self):
        N1 = self.N1
        i = np.arange(N1)
        iz, iy, ix = np.meshgrid(i, i, i, indexing="ij")
        on = (ix == 0) | (ix == N1 - 1) | (iy == 0) | (iy == N1 - 1) | (iz == 0) | (iz == N1 - 1)
        return np.nonzero(on.ravel())[0].astype(np.int32)
