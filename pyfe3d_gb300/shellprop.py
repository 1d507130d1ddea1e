"""Shell and beam property records (host side).

Restates the property objects of ``pyfe3d/shellprop.pyx`` and
``pyfe3d/beamprop.pyx`` that the element methods read: the laminate ABD/E
matrices, the shear correction factors and the density integrals.  They are
host-side inputs, as in the reference; the GPU kernels receive them flattened
into fixed-stride records (:func:`shell_record`, :func:`beam_record`).

Any object exposing the same attribute names (for instance a reference
``pyfe3d.shellprop.ShellProp``) is accepted wherever a property is expected.
"""
import math

import numpy as np

SHELL_PROP_STRIDE = 28
BEAM_PROP_STRIDE = 16
SHELL_FIELDS = ('A11', 'A12', 'A16', 'A22', 'A26', 'A66', 'B11', 'B12', 'B16', 'B22',
                'B26', 'B66', 'D11', 'D12', 'D16', 'D22', 'D26', 'D66', 'E44', 'E45',
                'E55', 'scf_k13', 'scf_k23', 'h', 'intrho', 'intrhoz', 'intrhoz2')
BEAM_FIELDS = ('A', 'E', 'G', 'Iyy', 'Izz', 'Iyz', 'J', 'Ay', 'Az', 'intrho', 'intrhoy',
               'intrhoz', 'intrhoy2', 'intrhoz2', 'intrhoyz')


def deg2rad(thetadeg):
    return thetadeg * 4 * math.atan(1.) / 180.


class MatLamina:
    """Orthotropic lamina material (pyfe3d/shellprop.pyx:43-196)."""

    def __init__(self):
        self.e1 = self.e2 = self.e3 = 0.
        self.g12 = self.g13 = self.g23 = 0.
        self.nu12 = self.nu21 = self.nu13 = self.nu31 = self.nu23 = self.nu32 = 0.
        self.rho = 0.

    def rebuild(self):
        """Plane-stress and 3D stiffness terms (shellprop.pyx:128-196)."""
        e1, e2, e3 = self.e1, self.e2, self.e3
        nu12, nu21, nu13, nu31, nu23, nu32 = (self.nu12, self.nu21, self.nu13, self.nu31,
                                              self.nu23, self.nu32)
        den = 1 - nu12 * nu21 - nu13 * nu31 - nu23 * nu32 - nu12 * nu23 * nu31 - nu13 * nu21 * nu32
        self.q11 = e1 * (1 - nu23 * nu32) / den
        self.q12 = e1 * (nu21 + nu23 * nu31) / den
        self.q22 = e2 * (1 - nu13 * nu31) / den
        self.q66 = self.g12
        self.q44 = self.g23
        self.q55 = self.g13


class Lamina:
    """One ply with its rotated plane-stress stiffness (shellprop.pyx:278-341)."""

    def __init__(self):
        self.h = 0.
        self.thetadeg = 0.
        self.matlamina = None

    def rebuild(self):
        t = deg2rad(self.thetadeg)
        self.cost = math.cos(t)
        self.sint = math.sin(t)
        cos2, cos3, cos4 = self.cost ** 2, self.cost ** 3, self.cost ** 4
        sin2, sin3, sin4 = self.sint ** 2, self.sint ** 3, self.sint ** 4
        sincos = self.sint * self.cost
        m = self.matlamina
        q11 = m.e1 / (1 - m.nu12 * m.nu21)
        q12 = m.nu12 * m.e2 / (1 - m.nu12 * m.nu21)
        q22 = m.e2 / (1 - m.nu12 * m.nu21)
        q44 = m.g23
        q55 = m.g13
        q66 = m.g12
        self.q11L = q11 * cos4 + 2 * (q12 + 2 * q66) * sin2 * cos2 + q22 * sin4
        self.q12L = (q11 + q22 - 4 * q66) * sin2 * cos2 + q12 * (sin4 + cos4)
        self.q22L = q11 * sin4 + 2 * (q12 + 2 * q66) * sin2 * cos2 + q22 * cos4
        self.q16L = (q11 - q12 - 2 * q66) * self.sint * cos3 + (q12 - q22 + 2 * q66) * sin3 * self.cost
        self.q26L = (q11 - q12 - 2 * q66) * sin3 * self.cost + (q12 - q22 + 2 * q66) * self.sint * cos3
        self.q66L = (q11 + q22 - 2 * q12 - 2 * q66) * sin2 * cos2 + q66 * (sin4 + cos4)
        self.q44L = q44 * cos2 + q55 * sin2
        self.q45L = (q55 - q44) * sincos
        self.q55L = q55 * cos2 + q44 * sin2


class ShellProp:
    """Laminate properties read by Quad4 (pyfe3d/shellprop.pyx:344-621)."""

    def __init__(self):
        self.h = 0.
        self.offset = 0.
        self.e1 = self.e2 = self.g12 = self.nu12 = self.nu21 = 0.
        self.scf_k13 = 5 / 6.
        self.scf_k23 = 5 / 6.
        self.intrho = self.intrhoz = self.intrhoz2 = 0.
        for f in SHELL_FIELDS[:21]:
            setattr(self, f, 0.)
        self.plies = []
        self.stack = []

    @property
    def A(self):
        return np.array([[self.A11, self.A12, self.A16], [self.A12, self.A22, self.A26],
                         [self.A16, self.A26, self.A66]])

    @property
    def B(self):
        return np.array([[self.B11, self.B12, self.B16], [self.B12, self.B22, self.B26],
                         [self.B16, self.B26, self.B66]])

    @property
    def D(self):
        return np.array([[self.D11, self.D12, self.D16], [self.D12, self.D22, self.D26],
                         [self.D16, self.D26, self.D66]])

    @property
    def E(self):
        return np.array([[self.E44, self.E45], [self.E45, self.E55]])

    @property
    def ABD(self):
        return np.block([[self.A, self.B], [self.B, self.D]])

    @property
    def ABDE(self):
        out = np.zeros((8, 8))
        out[:6, :6] = self.ABD
        out[6:, 6:] = self.E
        return out

    def calc_constitutive_matrix(self):
        """Ply integration of ABD, E and the density integrals (shellprop.pyx:568-621)."""
        self.h = sum(p.h for p in self.plies)
        h0 = -self.h / 2. + self.offset
        acc = dict.fromkeys(SHELL_FIELDS[:21], 0.)
        rho0 = rho1 = rho2 = 0.
        for ply in self.plies:
            hk_1 = h0
            h0 += ply.h
            hk = h0
            rho = ply.matlamina.rho
            rho0 += rho * (hk - hk_1)
            rho1 += rho * (hk * hk / 2. - hk_1 * hk_1 / 2.)
            rho2 += rho * (hk * hk * hk / 3. - hk_1 * hk_1 * hk_1 / 3.)
            d1 = hk - hk_1
            d2 = hk * hk - hk_1 * hk_1
            d3 = hk * hk * hk - hk_1 * hk_1 * hk_1
            for ij, q in (('11', ply.q11L), ('12', ply.q12L), ('16', ply.q16L),
                          ('22', ply.q22L), ('26', ply.q26L), ('66', ply.q66L)):
                acc['A' + ij] += q * d1
                acc['B' + ij] += 1 / 2. * q * d2
                acc['D' + ij] += 1 / 3. * q * d3
            acc['E44'] += ply.q44L * d1
            acc['E45'] += ply.q45L * d1
            acc['E55'] += ply.q55L * d1
        for k, v in acc.items():
            setattr(self, k, v)
        self.intrho, self.intrhoz, self.intrhoz2 = rho0, rho1, rho2

    def calc_scf(self):
        """Vlachoutsis shear correction factors (shellprop.pyx:485-549)."""
        D1 = R1 = den1 = D2 = R2 = den2 = 0.
        offset = self.offset
        zbot = -self.h / 2. + offset
        z1 = zbot
        for ply in self.plies:
            z2 = z1 + ply.h
            t = deg2rad(ply.thetadeg)
            m = ply.matlamina
            e1 = m.e1 * np.cos(t) + m.e2 * np.sin(t)
            e2 = m.e2 * np.cos(t) + m.e1 * np.sin(t)
            nu12 = m.nu12 * np.cos(t) + m.nu21 * np.sin(t)
            nu21 = m.nu21 * np.cos(t) + m.nu12 * np.sin(t)
            poly = (15 * offset * z1 ** 4 + 30 * offset * z1 ** 2 * zbot * (2 * offset - zbot)
                    - 15 * offset * z2 ** 4 + 30 * offset * z2 ** 2 * zbot * (-2 * offset + zbot)
                    - 3 * z1 ** 5 + 10 * z1 ** 3 * (-2 * offset ** 2 - 2 * offset * zbot + zbot ** 2)
                    - 15 * z1 * zbot ** 2 * (4 * offset ** 2 - 4 * offset * zbot + zbot ** 2)
                    + 3 * z2 ** 5 + 10 * z2 ** 3 * (2 * offset ** 2 + 2 * offset * zbot - zbot ** 2)
                    + 15 * z2 * zbot ** 2 * (4 * offset ** 2 - 4 * offset * zbot + zbot ** 2))
            D1 += e1 / (1 - nu12 * nu21)
            R1 += D1 * ((z2 - offset) ** 3 / 3. - (z1 - offset) ** 3 / 3.)
            den1 += m.g13 * ply.h * (self.h / ply.h) * D1 ** 2 * poly / (60 * m.g13)
            D2 += e2 / (1 - nu12 * nu21)
            R2 += D2 * ((z2 - offset) ** 3 / 3. - (z1 - offset) ** 3 / 3.)
            den2 += m.g23 * ply.h * (self.h / ply.h) * D2 ** 2 * poly / (60 * m.g23)
            z1 = z2
        self.scf_k13 = R1 ** 2 / den1
        self.scf_k23 = R2 ** 2 / den2

    def calc_equivalent_properties(self):
        """Equivalent laminate moduli (shellprop.pyx:551-566)."""
        AI = np.linalg.inv(self.ABD)
        a11, a12, a22, a33 = AI[0, 0], AI[0, 1], AI[1, 1], AI[2, 2]
        self.e1 = 1. / (self.h * a11)
        self.e2 = 1. / (self.h * a22)
        self.g12 = 1. / (self.h * a33)
        self.nu12 = -a12 / a11
        self.nu21 = -a12 / a22


class BeamProp:
    """Beam cross-section record (pyfe3d/beamprop.pyx:15-93), all fields zero."""

    def __init__(self):
        for f in BEAM_FIELDS:
            setattr(self, f, 0.)


def shell_record(prop):
    """Flatten a ShellProp-like object into one FE3D_SHELL_PROP_STRIDE record."""
    rec = np.zeros(SHELL_PROP_STRIDE)
    for i, f in enumerate(SHELL_FIELDS):
        rec[i] = float(getattr(prop, f))
    return rec


def beam_record(prop):
    rec = np.zeros(BEAM_PROP_STRIDE)
    for i, f in enumerate(BEAM_FIELDS):
        rec[i] = float(getattr(prop, f))
    return rec


def shell_records(props):
    return np.stack([shell_record(p) for p in props]) if len(props) else np.zeros((0, SHELL_PROP_STRIDE))


def beam_records(props):
    return np.stack([beam_record(p) for p in props]) if len(props) else np.zeros((0, BEAM_PROP_STRIDE))


def isotropic_plate_records(thickness, E, nu, rho=0., offset=0., calc_scf=True):
    """Vectorised ``isotropic_plate`` for arrays of thickness/E/nu/rho.

    Returns an (n, FE3D_SHELL_PROP_STRIDE) array whose rows equal
    ``shell_record(isotropic_plate(thickness[i], E[i], nu[i], ...))``: the same
    single-ply integration (shellprop.pyx:568-621) and shear correction
    (shellprop.pyx:485-549) evaluated with numpy over all entries.
    """
    h, E, nu, rho, offset = np.broadcast_arrays(*(np.asarray(v, dtype=np.float64)
                                                  for v in (thickness, E, nu, rho, offset)))
    n = h.shape[0] if h.ndim else 1
    h, E, nu, rho, offset = (np.atleast_1d(v).astype(np.float64) for v in (h, E, nu, rho, offset))
    g = E / (2 * (1 + nu))
    nu21 = nu * E / E
    q11 = E / (1 - nu * nu21)
    q12 = nu * E / (1 - nu * nu21)
    q22 = E / (1 - nu * nu21)
    # single ply at 0 degrees: cos = 1, sin = 0 (shellprop.pyx:303-341)
    q11L = q11 * 1. + 2 * (q12 + 2 * g) * 0. + q22 * 0.
    q12L = (q11 + q22 - 4 * g) * 0. + q12 * (0. + 1.)
    q22L = q11 * 0. + 2 * (q12 + 2 * g) * 0. + q22 * 1.
    q16L = (q11 - q12 - 2 * g) * 0. + (q12 - q22 + 2 * g) * 0.
    q26L = q16L.copy()
    q66L = (q11 + q22 - 2 * q12 - 2 * g) * 0. + g * (0. + 1.)
    q44L = g * 1. + g * 0.
    q45L = (g - g) * 0.
    q55L = g * 1. + g * 0.
    hk_1 = -h / 2. + offset
    hk = hk_1 + h
    d1 = hk - hk_1
    d2 = hk * hk - hk_1 * hk_1
    d3 = hk * hk * hk - hk_1 * hk_1 * hk_1
    rec = np.zeros((n, SHELL_PROP_STRIDE))
    for i, q in enumerate((q11L, q12L, q16L, q22L, q26L, q66L)):
        rec[:, i] = q * d1
        rec[:, 6 + i] = 1 / 2. * q * d2
        rec[:, 12 + i] = 1 / 3. * q * d3
    rec[:, 18] = q44L * d1
    rec[:, 19] = q45L * d1
    rec[:, 20] = q55L * d1
    if calc_scf:
        zbot = -h / 2. + offset
        z1, z2 = zbot, zbot + h
        D1 = E / (1 - nu * nu21)
        poly = (15 * offset * z1 ** 4 + 30 * offset * z1 ** 2 * zbot * (2 * offset - zbot)
                - 15 * offset * z2 ** 4 + 30 * offset * z2 ** 2 * zbot * (-2 * offset + zbot)
                - 3 * z1 ** 5 + 10 * z1 ** 3 * (-2 * offset ** 2 - 2 * offset * zbot + zbot ** 2)
                - 15 * z1 * zbot ** 2 * (4 * offset ** 2 - 4 * offset * zbot + zbot ** 2)
                + 3 * z2 ** 5 + 10 * z2 ** 3 * (2 * offset ** 2 + 2 * offset * zbot - zbot ** 2)
                + 15 * z2 * zbot ** 2 * (4 * offset ** 2 - 4 * offset * zbot + zbot ** 2))
        R1 = D1 * ((z2 - offset) ** 3 / 3. - (z1 - offset) ** 3 / 3.)
        den1 = g * h * (h / h) * D1 ** 2 * poly / (60 * g)
        scf = R1 ** 2 / den1
        rec[:, 21] = scf
        rec[:, 22] = scf
    else:
        rec[:, 21] = 5 / 6.
        rec[:, 22] = 5 / 6.
    rec[:, 23] = h
    rec[:, 24] = rho * d1
    rec[:, 25] = rho * (hk * hk / 2. - hk_1 * hk_1 / 2.)
    rec[:, 26] = rho * (hk * hk * hk / 3. - hk_1 * hk_1 * hk_1 / 3.)
    return rec


def isotropic_plate_records_device(thickness, E, nu, rho=0., offset=0., calc_scf=True):
    """``isotropic_plate_records`` computed on the GPU (one thread per record;
    fe3d_isotropic_plate_records): a CUDA tensor (n, 28).  Scalars broadcast
    against the arrays, whose common length is n."""
    from . import _lib
    torch = _lib.torch_mod()
    lib = _lib.load()
    args = []
    n = 1
    for v in (thickness, E, nu, rho, offset):
        t = _lib.to_device(np.atleast_1d(np.asarray(v, dtype=np.float64)) if not _lib.is_cuda_tensor(v) else v,
                           np.float64).reshape(-1)
        n = max(n, t.numel())
        args.append(t)
    for t in args:
        if t.numel() not in (1, n):
            raise ValueError('property arrays must have one entry or n entries')
    out = torch.empty((n, SHELL_PROP_STRIDE), dtype=torch.float64, device=args[0].device)
    flat = []
    for t in args:
        flat += [_lib.ptr(t), 1 if t.numel() == n and n > 1 else 0]
    rc = lib.fe3d_isotropic_plate_records(n, *flat, int(bool(calc_scf)), _lib.ptr(out), _lib.stream_ptr())
    _lib.check(rc, 'fe3d_isotropic_plate_records')
    return out



def _lamina_constants(lp):
    """The six lamina constants E11 E22 nu12 G12 G13 G23 of a 2-, 6- or
    9-tuple, as read_laminaprop reads them (shellprop_utils.py:13-93)."""
    lp = tuple(lp)
    if len(lp) == 2:
        e, nu = lp
        g = e / (2 * (1 + nu))
        return (e, e, nu, g, g, g)
    if len(lp) in (6, 9):
        return tuple(lp[:6])
    raise ValueError('Invalid entry for laminaprop: ' + str(lp))


def laminate_records_device(stack, plyt, laminaprop, rho=0., offset=0., calc_scf=True):
    """``laminated_plate`` records computed on the GPU (one thread per record;
    fe3d_laminate_records): a CUDA tensor (n, 28).

    ``stack`` (ply angles in degrees), ``plyt`` and ``rho`` are arrays of
    shape (nply,) shared by every record or (n, nply) per record (scalars
    broadcast to every ply); ``laminaprop`` is one lamina tuple, one per ply
    (nply, k) or one per ply and record (n, nply, k), k = 2, 6 or 9;
    ``offset`` a scalar or (n,)."""
    from . import _lib
    torch = _lib.torch_mod()
    lib = _lib.load()
    th = np.asarray(stack, dtype=np.float64)
    nply = th.shape[-1]
    pt = np.asarray(plyt, dtype=np.float64)
    if pt.ndim == 0:
        pt = np.full(nply, float(pt))
    rh = np.asarray(rho, dtype=np.float64)
    if rh.ndim == 0:
        rh = np.full(nply, float(rh))
    lp = np.asarray(laminaprop, dtype=np.float64)
    if lp.ndim == 1:
        lp = np.tile(np.array(_lamina_constants(lp)), (nply, 1))
    elif lp.ndim == 2:
        lp = np.array([_lamina_constants(r) for r in lp])
    else:
        lp = np.array([[_lamina_constants(r) for r in rec] for rec in lp])
    off = np.atleast_1d(np.asarray(offset, dtype=np.float64))
    n = max(a.shape[0] if a.ndim == 2 else 1 for a in (th, pt, rh))
    n = max(n, lp.shape[0] if lp.ndim == 3 else 1, off.shape[0])
    args = []
    for a, per in ((th, nply), (pt, nply), (lp, 6 * nply), (rh, nply)):
        shared = a.ndim == (2 if a is lp else 1)
        t = _lib.to_device(np.ascontiguousarray(a).reshape(-1), np.float64)
        if not shared and t.numel() != n * per:
            raise ValueError('per-record ply arrays must describe every record')
        args += [_lib.ptr(t), 0 if shared else per]
        _lib.keep(t)
    ot = _lib.to_device(off, np.float64)
    if ot.numel() not in (1, n):
        raise ValueError('offset must be a scalar or one per record')
    _lib.keep(ot)
    out = torch.empty((n, SHELL_PROP_STRIDE), dtype=torch.float64, device=ot.device)
    rc = lib.fe3d_laminate_records(n, nply, args[0], args[1], args[2], args[3], args[4], args[5], args[6], args[7],
                                   _lib.ptr(ot), 1 if ot.numel() == n and n > 1 else 0, int(bool(calc_scf)),
                                   _lib.ptr(out), _lib.stream_ptr())
    _lib.check(rc, 'fe3d_laminate_records')
    return out
