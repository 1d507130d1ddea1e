"""Seeded synthetic meshes of the plate and panel shapes the path is measured on.

Node numbering follows the reference tests (tests/test_quad4_static_point_load.py:34-40):
``nids.reshape(nx, ny)`` with the x index slow, elements n1..n4 counter-clockwise.
"""
import numpy as np

from .shellprop import BEAM_PROP_STRIDE, isotropic_plate_records

DOF = 6


class PlateMesh:
    """Structured quadrilateral mesh of a rectangular plate in the XY plane."""

    def __init__(self, nx, ny, a, b, perturb=0.0, seed=None):
        self.nx, self.ny, self.a, self.b = nx, ny, a, b
        xt = np.linspace(0, a, nx)
        yt = np.linspace(0, b, ny)
        xm, ym = np.meshgrid(xt, yt, indexing='ij')
        X = xm.ravel().copy()
        Y = ym.ravel().copy()
        self.edge = (np.isclose(X, 0) | np.isclose(X, a) | np.isclose(Y, 0) | np.isclose(Y, b))
        if perturb > 0:
            rng = np.random.default_rng(seed)
            dx = a / (nx - 1)
            dy = b / (ny - 1)
            inner = ~self.edge
            X[inner] += rng.uniform(-perturb, perturb, inner.sum()) * dx
            Y[inner] += rng.uniform(-perturb, perturb, inner.sum()) * dy
        self.ncoords = np.stack([X, Y, np.zeros_like(X)], axis=1)
        self.x = self.ncoords.ravel()
        nids = np.arange(nx * ny).reshape(nx, ny)
        self.nids = nids
        n1 = nids[:-1, :-1].ravel()
        n2 = nids[1:, :-1].ravel()
        n3 = nids[1:, 1:].ravel()
        n4 = nids[:-1, 1:].ravel()
        self.conn = np.stack([n1, n2, n3, n4], axis=1)
        self.cdof = (DOF * self.conn).astype(np.int64)
        self.E = self.conn.shape[0]
        self.nnodes = nx * ny
        self.N = DOF * self.nnodes

    def init_k(self, size, start=0):
        return start + size * np.arange(self.E, dtype=np.int64)

    def bc_mask(self, dofs):
        """Boolean mask of constrained DOFs: the given DOFs of every edge node."""
        bk = np.zeros(self.N, dtype=bool)
        for d in dofs:
            bk[d::DOF] = self.edge
        return bk

    def centre_node(self):
        return int(self.nids[self.nx // 2, self.ny // 2])


def config1():
    """21x21-node simply supported isotropic plate, -1000 N at the centre."""
    m = PlateMesh(21, 21, 1.0, 1.0)
    props = isotropic_plate_records(0.005, 70e9, 0.33)
    bk = m.bc_mask((0, 1, 2))
    f = np.zeros(m.N)
    f[DOF * m.centre_node() + 2] = -1000.
    return m, props, None, bk, f


def config2(n=1001, seed=2, thick_seed=3):
    """n x n-node clamped plate on 2.0 x 2.0 m, interior nodes perturbed by up
    to 10% of the element size, log-normal thickness per element
    (median 0.005 m, sigma 0.3), -1 N on w at every free node."""
    m = PlateMesh(n, n, 2.0, 2.0, perturb=0.1, seed=seed)
    rng = np.random.default_rng(thick_seed)
    h = 0.005 * np.exp(0.3 * rng.standard_normal(m.E))
    props = isotropic_plate_records(h, 70e9, 0.33)
    pid = np.arange(m.E, dtype=np.int32)
    bk = m.bc_mask(range(6))
    f = np.zeros(m.N)
    f[2::DOF] = -1.
    f[bk] = 0.
    return m, props, pid, bk, f


def stringer_records(E=70e9, nu=0.33, height=0.02, thickness=0.004, rho=0.):
    """Rectangular blade stringer: height along the element z axis (normal to
    the skin when vxy lies in the skin plane), thickness along y.  J follows
    the reference tests' convention J = Iyy + Izz."""
    rec = np.zeros(BEAM_PROP_STRIDE)
    A = height * thickness
    Iyy = thickness * height ** 3 / 12.   # int z^2 dA
    Izz = height * thickness ** 3 / 12.   # int y^2 dA
    G = E / (2 * (1 + nu))
    rec[0:9] = [A, E, G, Iyy, Izz, 0., Iyy + Izz, 0., 0.]
    rec[9] = rho * A
    rec[12] = rho * Izz
    rec[13] = rho * Iyy
    return rec


class StiffenedPanel:
    """Quad4 skin of nel x nel elements on a 1.0 x 1.0 m plate, laminated
    [0/45/-45/90]s (ply 0.125 mm, E11=142.5e9, E22=8.7e9, nu12=0.28,
    G12=G13=G23=5.1e9), with 9 BeamC stringers along x at y = 0.1 k
    (k = 1..9) sharing the skin nodes (vxy = (0, 1, 0), blade 0.02 x 0.004 m,
    E = 70e9, nu = 0.33).  Simply supported: w = 0 on every edge, u = 0 on
    x = 0, v = 0 on y = 0; -1 N on u at each node of the x = 1 edge and
    -0.1 N on w at every free node."""

    def __init__(self, nel=500):
        from .shellprop import shell_record
        from .shellprop_utils import laminated_plate
        if nel % 10:
            raise ValueError('nel must be a multiple of 10 (stringers at y = 0.1 k)')
        n = nel + 1
        self.skin = PlateMesh(n, n, 1.0, 1.0)
        lam = laminated_plate([0, 45, -45, 90, 90, -45, 45, 0], plyt=0.000125,
                              laminaprop=(142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9))
        self.shell_props = shell_record(lam)[None, :]
        rows = [nel // 10 * k for k in range(1, 10)]
        nids = self.skin.nids  # [ix, iy]
        n1 = np.concatenate([nids[:-1, r] for r in rows])
        n2 = np.concatenate([nids[1:, r] for r in rows])
        self.beam_cdof = (DOF * np.stack([n1, n2], 1)).astype(np.int64)
        self.beam_props = stringer_records()[None, :]
        self.vxy = np.array([0., 1., 0.])
        self.Eq = self.skin.E
        self.Eb = self.beam_cdof.shape[0]
        self.N = self.skin.N
        X, Y = self.skin.ncoords[:, 0], self.skin.ncoords[:, 1]
        bk = np.zeros(self.N, dtype=bool)
        bk[2::DOF] = self.skin.edge
        bk[0::DOF] |= np.isclose(X, 0.)
        bk[1::DOF] |= np.isclose(Y, 0.)
        self.bk = bk
        f = np.zeros(self.N)
        f[0::DOF][np.isclose(X, 1.)] = -1.
        f[2::DOF] = -0.1
        f[bk] = 0.
        self.f = f

    def coo_sizes(self):
        return 576 * self.Eq, 144 * self.Eb


def config3(nel=500):
    return StiffenedPanel(nel)


class BatchedPlates:
    """Many independent isotropic Quad4 plates numbered one after another in
    one global system (block-diagonal stiffness).

    Per plate (seeded): nx and ny elements per side uniform integers in
    [nmin, nmax] (nx + 1 by ny + 1 nodes),
    side lengths uniform in [0.5, 2.0] m, E uniform in [50e9, 210e9] Pa, nu in
    [0.25, 0.35], h in [0.001, 0.02] m, edges simply supported (u, v, w fixed)
    or clamped (all six DOFs fixed) at random, -1000 N on w at the centre
    node.  Attributes follow :class:`PlateMesh` for the whole system plus
    per-plate offsets (``node0``, ``dof0``, ``elem0``) and ``inst_of_dof``.
    """

    def __init__(self, nplates=1024, nmin=8, nmax=256, seed=4):
        rng = np.random.default_rng(seed)
        P = int(nplates)
        nx = rng.integers(nmin, nmax + 1, P)
        ny = rng.integers(nmin, nmax + 1, P)
        a = rng.uniform(0.5, 2.0, P)
        b = rng.uniform(0.5, 2.0, P)
        Emod = rng.uniform(50e9, 210e9, P)
        nu = rng.uniform(0.25, 0.35, P)
        h = rng.uniform(0.001, 0.02, P)
        clamped = rng.integers(0, 2, P).astype(bool)
        self._build(nx, ny, a, b, Emod, nu, h, clamped)

    def _build(self, nx, ny, a, b, Emod, nu, h, clamped):
        self.nx, self.ny, self.a, self.b = nx, ny, a, b
        self.Emod, self.nu, self.h, self.clamped = Emod, nu, h, clamped
        P = self.P = len(nx)
        nn = (self.nx + 1) * (self.ny + 1)
        ne = self.nx * self.ny
        self.node0 = np.concatenate([[0], np.cumsum(nn)]).astype(np.int64)
        self.elem0 = np.concatenate([[0], np.cumsum(ne)]).astype(np.int64)
        self.dof0 = DOF * self.node0
        self.nnodes = int(self.node0[-1])
        self.E = int(self.elem0[-1])
        self.N = DOF * self.nnodes
        self.props = isotropic_plate_records(self.h, self.Emod, self.nu)
        x = np.empty((self.nnodes, 3))
        cdof = np.empty((self.E, 4), dtype=np.int64)
        pid = np.empty(self.E, dtype=np.int32)
        bk = np.zeros(self.N, dtype=bool)
        f = np.zeros(self.N)
        for i in range(P):
            m = PlateMesh(int(self.nx[i]) + 1, int(self.ny[i]) + 1, self.a[i], self.b[i])
            n0, e0, d0 = self.node0[i], self.elem0[i], self.dof0[i]
            x[n0:n0 + m.nnodes] = m.ncoords
            cdof[e0:e0 + m.E] = m.cdof + d0
            pid[e0:e0 + m.E] = i
            bk[d0:d0 + m.N] = m.bc_mask(range(6) if self.clamped[i] else (0, 1, 2))
            f[d0 + DOF * m.centre_node() + 2] = -1000.
        f[bk] = 0.
        self.x = x.ravel()
        self.cdof = cdof
        self.pid = pid
        self.bk = bk
        self.f = f
        self.inst_of_dof = np.repeat(np.arange(P, dtype=np.int32), DOF * nn)

    def subset(self, idx):
        """The plates idx (in that order) as a batch of their own."""
        idx = np.asarray(idx)
        sub = BatchedPlates.__new__(BatchedPlates)
        sub._build(self.nx[idx], self.ny[idx], self.a[idx], self.b[idx], self.Emod[idx], self.nu[idx],
                   self.h[idx], self.clamped[idx])
        return sub

    def plate(self, i):
        """Plate i alone (its own numbering, one property record)."""
        return self.subset([i])

    def init_k(self, size, start=0):
        return start + size * np.arange(self.E, dtype=np.int64)

    def plate_dofs(self, i):
        return slice(int(self.dof0[i]), int(self.dof0[i + 1]))


def config4(nplates=1024, nmin=8, nmax=256, seed=4):
    return BatchedPlates(nplates, nmin, nmax, seed)


def gaussian_random_field(nx, ny, dx, corr_length, rng):
    """Zero-mean, unit-variance Gaussian random field on an nx x ny grid of
    spacing dx with squared-exponential covariance exp(-d^2 / (2 l^2)),
    sampled by filtering white noise in Fourier space (periodic)."""
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=dx)
    k2 = kx[:, None] ** 2 + ky[None, :] ** 2
    amp = np.exp(-0.25 * k2 * corr_length ** 2)  # sqrt of the Gaussian spectrum
    g = np.real(np.fft.ifft2(np.fft.fft2(rng.standard_normal((nx, ny))) * amp))
    g -= g.mean()
    sd = g.std()
    return g / sd if sd > 0 else g


class RandomFieldPlate(PlateMesh):
    """Square 1.0 x 1.0 m isotropic plate of nel x nel Quad4 elements
    (E = 70e9 Pa, nu = 0.33) whose thickness per element is log-normal with
    median 0.005 m and sigma 0.5 drawn from a Gaussian random field of
    correlation length 0.1 m; edges simply supported (u, v, w fixed) or
    clamped at random; seeded normal random loads on w at every free node."""

    def __init__(self, nel, seed=0):
        super().__init__(nel + 1, nel + 1, 1.0, 1.0)
        rng = np.random.default_rng(seed)
        g = gaussian_random_field(nel, nel, 1.0 / nel, 0.1, rng)
        self.h = 0.005 * np.exp(0.5 * g.ravel())
        self.props = isotropic_plate_records(self.h, 70e9, 0.33)
        self.pid = np.arange(self.E, dtype=np.int32)
        self.clamped = bool(rng.integers(0, 2))
        self.bk = self.bc_mask(range(6) if self.clamped else (0, 1, 2))
        f = np.zeros(self.N)
        f[2::DOF] = rng.standard_normal(self.nnodes)
        f[self.bk] = 0.
        self.f = f


def config5_training_plates(count=200, nel_min=64, nel_max=256, seed=5):
    """Training plates: square meshes of nel_min^2 .. nel_max^2 elements."""
    rng = np.random.default_rng(seed)
    return [RandomFieldPlate(int(rng.integers(nel_min, nel_max + 1)), seed=int(rng.integers(1 << 30)))
            for _ in range(count)]
