"""Generate the golden fixtures by running the reference implementation.

The reference (pyfe3d, Cython) cannot travel to the GPU host, so its outputs
on seeded inputs are frozen here as small ``.npz`` files.  Run from the
repository root in a container where the reference sources are available:

    python tests/golden/make_golden.py --ref /path/to/pyfe3d/checkout

(or set PYFE3D_REF to that path instead of passing --ref).

If ``pyfe3d`` is not importable, the reference checkout is copied to a
temporary directory and its extensions are built in place there (the
checkout itself is never written to).

Fixtures written next to this script:
  quad4_elements.npz   frames, probes, KC0/KG/M triplets, internal forces and
                       KG of given stress resultants of single Quad4s
  beamc_elements.npz   the same for BeamC (KC0/KG/M, internal forces)
  shellprop.npz        ABD/E, shear correction and density integrals
  plate_static.npz     the 21x21-node point-load plate solved with spsolve
  tria3r_elements.npz  frames, probes, KC0/KG/M triplets, internal forces and
                       KG of given stress resultants of single Tria3Rs
  quad4r_elements.npz  the same for Quad4R (hourglass factors, K6ROT varied)
  tria3r_static.npz    the 7x11-node Tria3R point-load plate of the
                       reference tests solved with spsolve
"""
import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

SHELL_FIELDS = ('A11', 'A12', 'A16', 'A22', 'A26', 'A66', 'B11', 'B12', 'B16', 'B22',
                'B26', 'B66', 'D11', 'D12', 'D16', 'D22', 'D26', 'D66', 'E44', 'E45',
                'E55', 'scf_k13', 'scf_k23', 'h', 'intrho', 'intrhoz', 'intrhoz2')
BEAM_FIELDS = ('A', 'E', 'G', 'Iyy', 'Izz', 'Iyz', 'J', 'Ay', 'Az', 'intrho', 'intrhoy',
               'intrhoz', 'intrhoy2', 'intrhoz2', 'intrhoyz')


def import_reference(ref):
    try:
        import pyfe3d  # noqa: F401
        return
    except ImportError:
        pass
    build = os.path.join(tempfile.gettempdir(), 'pyfe3d_golden_build')
    if not os.path.exists(os.path.join(build, 'pyfe3d', 'quad4.pyx')):
        shutil.rmtree(build, ignore_errors=True)
        shutil.copytree(ref, build)
        for root, dirs, files in os.walk(build):
            for f in files + dirs:
                os.chmod(os.path.join(root, f), 0o755)
    subprocess.run([sys.executable, 'setup.py', 'build_ext', '--inplace', '-j', '8'],
                   cwd=build, check=True, capture_output=True)
    sys.path.insert(0, build)


def shell_rec(p):
    return np.array([float(getattr(p, f)) for f in SHELL_FIELDS] + [0.])


def beam_rec(p):
    return np.array([float(getattr(p, f)) for f in BEAM_FIELDS] + [0.])


def make_shell_props():
    from pyfe3d.shellprop_utils import isotropic_plate, laminated_plate
    lam = (142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9)
    specs = [
        ('iso_thin', lambda: isotropic_plate(0.005, 70e9, 0.33)),
        ('iso_rho', lambda: isotropic_plate(0.01, 70e9, 0.3, rho=2700)),
        ('iso_thick', lambda: isotropic_plate(0.8, 70e9, 0.3, rho=2700)),
        ('iso_offset', lambda: isotropic_plate(0.004, 200e9, 0.3, offset=0.001, rho=7800)),
        ('lam_quasi', lambda: laminated_plate([0, 45, -45, 90, 90, -45, 45, 0], plyt=0.000125,
                                              laminaprop=lam)),
        ('lam_unsym', lambda: laminated_plate([0, 45, -45, 90, 30], plyt=0.0011, laminaprop=lam,
                                              rho=1600, offset=0.001)),
        ('lam_iso2', lambda: laminated_plate([0, 90], plyt=0.002, laminaprop=(70e9, 0.33),
                                             rho=2700)),
        ('lam_noscf', lambda: laminated_plate([15, -15], plyt=0.001, laminaprop=lam,
                                              calc_scf=False)),
    ]
    names, recs, props = [], [], []
    for name, fn in specs:
        p = fn()
        names.append(name)
        recs.append(shell_rec(p))
        props.append(p)
    return names, np.array(recs), props


def quad4_cases(props, rng):
    from pyfe3d import Quad4, Quad4Probe, INT
    out = {k: [] for k in ('x', 'c', 'xmat', 'pid', 'u', 'R', 'm', 'xe', 'area', 'ue',
                           'KC0r', 'KC0c', 'KC0v', 'KGr', 'KGc', 'KGv', 'M0r', 'M0c', 'M0v',
                           'M1v', 'M2r', 'M2c', 'M2v', 'fint', 'finte', 'Nstress', 'KGsr', 'KGsc',
                           'KGsv')}
    # stress resultants for update_KG_given_stress from their own stream, so
    # the other fields keep their values
    rng_n = np.random.default_rng(7)
    ncase = 48
    for t in range(ncase):
        base = np.array([0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0.]) * rng.uniform(0.05, 2.0)
        jit = rng.uniform(-0.15, 0.15, 12) * np.abs(base).max()
        if t % 2 == 0:
            jit[2::3] = 0.  # flat in the XY plane
        x = (base + jit).reshape(4, 3)
        if t % 3 == 0:  # arbitrary 3D orientation and offset
            q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
            if np.linalg.det(q) < 0:
                q[:, 0] *= -1
            x = x @ q.T
        x = x + rng.uniform(-3, 3, 3)
        perm = rng.permutation(4)
        xg = np.zeros((4, 3))
        xg[perm] = x  # node i of the element sits at global node perm[i]
        c = 6 * perm
        pid = t % len(props)
        prop = props[pid]
        xmat = rng.normal(size=3) if t % 4 == 1 else np.full(3, np.nan)
        q4 = Quad4(Quad4Probe())
        q4.c1, q4.c2, q4.c3, q4.c4 = [int(v) for v in c]
        xf = xg.flatten()
        if np.isfinite(xmat).all():
            q4.update_rotation_matrix(xf, *xmat)
        else:
            q4.update_rotation_matrix(xf)
        q4.update_probe_xe(xf)
        u = rng.normal(size=24) * 1e-3
        q4.update_probe_ue(u)
        def coo(n):
            return np.zeros(n, INT), np.zeros(n, INT), np.zeros(n)
        KC0 = coo(576)
        q4.update_KC0(*KC0, prop)
        KG = coo(144)
        q4.update_KG(*KG, prop)
        M0, M1, M2 = coo(480), coo(480), coo(480)
        q4.update_M(*M0, prop, mtype=0)
        q4.update_M(*M1, prop, mtype=1)
        q4.update_M(*M2, prop, mtype=2)
        fint = np.zeros(24)
        q4.update_fint(fint, prop)
        finte = np.asarray(q4.probe.finte).copy()
        Ns = rng_n.normal(size=3) * 1e3
        KGs = coo(144)
        q4.update_KG_given_stress(float(Ns[0]), float(Ns[1]), float(Ns[2]), *KGs)
        out['x'].append(xf); out['c'].append(c); out['xmat'].append(xmat)
        out['pid'].append(pid); out['u'].append(u)
        out['R'].append([q4.r11, q4.r12, q4.r13, q4.r21, q4.r22, q4.r23, q4.r31, q4.r32, q4.r33])
        out['m'].append([q4.m11, q4.m12, q4.m21, q4.m22])
        out['xe'].append(np.asarray(q4.probe.xe).copy()); out['area'].append(q4.area)
        out['ue'].append(np.asarray(q4.probe.ue).copy())
        out['KC0r'].append(KC0[0]); out['KC0c'].append(KC0[1]); out['KC0v'].append(KC0[2])
        out['KGr'].append(KG[0]); out['KGc'].append(KG[1]); out['KGv'].append(KG[2])
        out['M0r'].append(M0[0]); out['M0c'].append(M0[1]); out['M0v'].append(M0[2])
        out['M1v'].append(M1[2])
        out['M2r'].append(M2[0]); out['M2c'].append(M2[1]); out['M2v'].append(M2[2])
        out['fint'].append(fint)
        out['finte'].append(finte); out['Nstress'].append(Ns)
        out['KGsr'].append(KGs[0]); out['KGsc'].append(KGs[1]); out['KGsv'].append(KGs[2])
    return {k: np.array(v) for k, v in out.items()}


def beamc_cases(rng):
    from pyfe3d import BeamC, BeamCProbe, INT
    from pyfe3d.beamprop import BeamProp
    out = {k: [] for k in ('x', 'c', 'vxy', 'prop', 'u', 'R', 'xe', 'length', 'ue',
                           'KC0r', 'KC0c', 'KC0v', 'KGr', 'KGc', 'KGv', 'KGv_only_r',
                           'M0r', 'M0c', 'M0v', 'M1r', 'M1c', 'M1v', 'finte', 'fint')}
    for t in range(32):
        x = rng.normal(size=(2, 3)) * rng.uniform(0.01, 2.0)
        vxy = rng.normal(size=3)
        perm = rng.permutation(2)
        xg = np.zeros((2, 3))
        xg[perm] = x
        c = 6 * perm
        bp = BeamProp()
        bp.A = 1e-3 * rng.uniform(0.5, 2)
        bp.E = rng.uniform(50e9, 210e9)
        bp.G = bp.E / 2 / (1 + rng.uniform(0.25, 0.35))
        bp.Iyy = 1e-7 * rng.uniform(0.5, 2)
        bp.Izz = 2e-7 * rng.uniform(0.5, 2)
        bp.Iyz = (1e-8 * rng.uniform(-1, 1)) if t % 2 else 0.
        bp.J = bp.Iyy + bp.Izz
        bp.Ay = (1e-5 * rng.uniform(-1, 1)) if t % 3 else 0.
        bp.Az = (1e-5 * rng.uniform(-1, 1)) if t % 3 else 0.
        rho = rng.uniform(1000, 8000)
        bp.intrho = rho * bp.A
        bp.intrhoy = rho * bp.Ay
        bp.intrhoz = rho * bp.Az
        bp.intrhoy2 = rho * bp.Izz
        bp.intrhoz2 = rho * bp.Iyy
        bp.intrhoyz = rho * bp.Iyz
        b = BeamC(BeamCProbe())
        b.c1, b.c2 = [int(v) for v in c]
        xf = xg.flatten()
        b.update_rotation_matrix(*vxy, xf)
        b.update_probe_xe(xf)
        u = rng.normal(size=12) * 1e-3
        b.update_probe_ue(u)
        def coo(n):
            return np.zeros(n, INT), np.zeros(n, INT), np.zeros(n)
        KC0 = coo(144)
        b.update_KC0(*KC0, bp)
        KG = coo(144)
        b.update_KG(*KG, bp, update_KGv_only=0)
        KGo = coo(144)
        b.update_KG(*KGo, bp, update_KGv_only=1)
        M0, M1 = coo(144), coo(144)
        b.update_M(*M0, bp, mtype=0)
        b.update_M(*M1, bp, mtype=1)
        fint = np.zeros(12)
        b.update_fint(fint, bp)
        finte = np.asarray(b.probe.finte).copy()
        out['x'].append(xf); out['c'].append(c); out['vxy'].append(vxy)
        out['prop'].append(beam_rec(bp)); out['u'].append(u)
        out['R'].append([b.r11, b.r12, b.r13, b.r21, b.r22, b.r23, b.r31, b.r32, b.r33])
        out['xe'].append(np.asarray(b.probe.xe).copy()); out['length'].append(b.length)
        out['ue'].append(np.asarray(b.probe.ue).copy())
        out['KC0r'].append(KC0[0]); out['KC0c'].append(KC0[1]); out['KC0v'].append(KC0[2])
        out['KGr'].append(KG[0]); out['KGc'].append(KG[1]); out['KGv'].append(KG[2])
        out['KGv_only_r'].append(KGo[0])
        out['M0r'].append(M0[0]); out['M0c'].append(M0[1]); out['M0v'].append(M0[2])
        out['M1r'].append(M1[0]); out['M1c'].append(M1[1]); out['M1v'].append(M1[2])
        out['finte'].append(finte); out['fint'].append(fint)
    return {k: np.array(v) for k, v in out.items()}


def plate_static():
    """The 21x21-node simply supported plate with a centre point load."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import spsolve
    from pyfe3d import Quad4, Quad4Data, Quad4Probe, INT, DOUBLE, DOF
    from pyfe3d.shellprop_utils import isotropic_plate
    data = Quad4Data()
    probe = Quad4Probe()
    nx = ny = 21
    a = b = 1.0
    xtmp = np.linspace(0, a, nx)
    ytmp = np.linspace(0, b, ny)
    xmesh, ymesh = np.meshgrid(xtmp, ytmp)
    ncoords = np.vstack((xmesh.T.flatten(), ymesh.T.flatten(), np.zeros(nx * ny))).T
    xf = ncoords.flatten()
    nids = np.arange(nx * ny).reshape(nx, ny)
    n1s = nids[:-1, :-1].flatten()
    n2s = nids[1:, :-1].flatten()
    n3s = nids[1:, 1:].flatten()
    n4s = nids[:-1, 1:].flatten()
    E = len(n1s)
    N = DOF * nx * ny
    KC0r = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=INT)
    KC0c = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=INT)
    KC0v = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=DOUBLE)
    prop = isotropic_plate(thickness=0.005, E=70e9, nu=0.33, calc_scf=True)
    for e, (n1, n2, n3, n4) in enumerate(zip(n1s, n2s, n3s, n4s)):
        q = Quad4(probe)
        q.c1, q.c2, q.c3, q.c4 = DOF * n1, DOF * n2, DOF * n3, DOF * n4
        q.init_k_KC0 = e * data.KC0_SPARSE_SIZE
        q.update_rotation_matrix(xf)
        q.update_probe_xe(xf)
        q.update_KC0(KC0r, KC0c, KC0v, prop)
    K = coo_matrix((KC0v, (KC0r, KC0c)), shape=(N, N)).tocsc()
    bk = np.zeros(N, dtype=bool)
    edge = (np.isclose(ncoords[:, 0], 0) | np.isclose(ncoords[:, 0], a) |
            np.isclose(ncoords[:, 1], 0) | np.isclose(ncoords[:, 1], b))
    for d in range(3):
        bk[d::DOF] = edge
    bu = ~bk
    f = np.zeros(N)
    centre = nids[nx // 2, ny // 2]
    f[DOF * centre + 2] = -1000.
    Kuu = K[bu, :][:, bu]
    u = np.zeros(N)
    u[bu] = spsolve(Kuu, f[bu])
    conn = np.stack([n1s, n2s, n3s, n4s], axis=1)
    return dict(x=xf, conn=conn, bk=bk, f=f, u=u, prop=shell_rec(prop),
                KC0v_first=KC0v[:8 * 576], KC0r_first=KC0r[:8 * 576],
                KC0c_first=KC0c[:8 * 576], Kdiag=K.diagonal(), nnz=K.nnz)


def _shell_geometry(rng, nn, t):
    """Nodes of one shell element: a jittered unit triangle / square, flat in
    the XY plane for even t, turned to an arbitrary 3D orientation for t % 3
    == 0, shifted, and scattered over global node slots."""
    if nn == 3:
        base = np.array([0, 0, 0, 1, 0, 0, 0.3, 0.9, 0.]) * rng.uniform(0.05, 2.0)
    else:
        base = np.array([0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0.]) * rng.uniform(0.05, 2.0)
    jit = rng.uniform(-0.15, 0.15, 3 * nn) * np.abs(base).max()
    if t % 2 == 0:
        jit[2::3] = 0.
    x = (base + jit).reshape(nn, 3)
    if t % 3 == 0:
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        if np.linalg.det(q) < 0:
            q[:, 0] *= -1
        x = x @ q.T
    x = x + rng.uniform(-3, 3, 3)
    perm = rng.permutation(nn)
    xg = np.zeros((nn, 3))
    xg[perm] = x
    return xg.flatten(), 6 * perm


def _coo(n):
    from pyfe3d import INT
    return np.zeros(n, INT), np.zeros(n, INT), np.zeros(n)


def tria3r_cases(props, rng):
    from pyfe3d import Tria3R, Tria3RProbe
    keys = ('x', 'c', 'xmat', 'pid', 'u', 'k6rot', 'alpha', 'R', 'm', 'xe', 'area', 'ue',
            'KC0r', 'KC0c', 'KC0v', 'KGr', 'KGc', 'KGv', 'M0r', 'M0c', 'M0v', 'M1v', 'M2r',
            'M2c', 'M2v', 'fint', 'finte', 'Nstress', 'KGsr', 'KGsc', 'KGsv')
    out = {k: [] for k in keys}
    for t in range(48):
        xf, c = _shell_geometry(rng, 3, t)
        pid = t % len(props)
        prop = props[pid]
        xmat = rng.normal(size=3) if t % 4 == 1 else np.full(3, np.nan)
        el = Tria3R(Tria3RProbe())
        el.c1, el.c2, el.c3 = [int(v) for v in c]
        el.K6ROT = float(rng.choice([100., 1e4, 3.7]))
        el.alpha_shear_locking = float(rng.choice([0.7, 0.2, 1.3]))
        if np.isfinite(xmat).all():
            el.update_rotation_matrix(xf, *xmat)
        else:
            el.update_rotation_matrix(xf)
        el.update_probe_xe(xf)
        u = rng.normal(size=18) * 1e-3
        el.update_probe_ue(u)
        KC0 = _coo(324)
        el.update_KC0(*KC0, prop)
        KG = _coo(81)
        el.update_KG(*KG, prop)
        M0, M1, M2 = _coo(270), _coo(270), _coo(270)
        el.update_M(*M0, prop, mtype=0)
        el.update_M(*M1, prop, mtype=1)
        el.update_M(*M2, prop, mtype=2)
        fint = np.zeros(18)
        el.update_fint(fint, prop)
        finte = np.asarray(el.probe.finte).copy()
        Ns = rng.normal(size=3) * 1e3
        KGs = _coo(81)
        el.update_KG_given_stress(float(Ns[0]), float(Ns[1]), float(Ns[2]), *KGs)
        vals = dict(x=xf, c=c, xmat=xmat, pid=pid, u=u, k6rot=el.K6ROT, alpha=el.alpha_shear_locking,
                    R=[el.r11, el.r12, el.r13, el.r21, el.r22, el.r23, el.r31, el.r32, el.r33],
                    m=[el.m11, el.m12, el.m21, el.m22], xe=np.asarray(el.probe.xe).copy(),
                    area=el.area, ue=np.asarray(el.probe.ue).copy(),
                    KC0r=KC0[0], KC0c=KC0[1], KC0v=KC0[2], KGr=KG[0], KGc=KG[1], KGv=KG[2],
                    M0r=M0[0], M0c=M0[1], M0v=M0[2], M1v=M1[2], M2r=M2[0], M2c=M2[1], M2v=M2[2],
                    fint=fint, finte=finte, Nstress=Ns, KGsr=KGs[0], KGsc=KGs[1], KGsv=KGs[2])
        for k in keys:
            out[k].append(vals[k])
    return {k: np.array(v) for k, v in out.items()}


def quad4r_cases(props, rng):
    from pyfe3d import Quad4R, Quad4RProbe
    keys = ('x', 'c', 'xmat', 'pid', 'u', 'k6rot', 'hg', 'R', 'm', 'xe', 'area', 'ue',
            'KC0r', 'KC0c', 'KC0v', 'KGr', 'KGc', 'KGv', 'M0v', 'M1v', 'M2v', 'fint', 'finte',
            'Nstress', 'KGsv')
    out = {k: [] for k in keys}
    for t in range(48):
        xf, c = _shell_geometry(rng, 4, t)
        pid = t % len(props)
        prop = props[pid]
        xmat = rng.normal(size=3) if t % 4 == 1 else np.full(3, np.nan)
        el = Quad4R(Quad4RProbe())
        el.c1, el.c2, el.c3, el.c4 = [int(v) for v in c]
        el.K6ROT = float(rng.choice([100., 1e4, 3.7]))
        hg = np.ones(5) if t % 3 else rng.uniform(0.1, 3.0, 5)
        if np.isfinite(xmat).all():
            el.update_rotation_matrix(xf, *xmat)
        else:
            el.update_rotation_matrix(xf)
        el.update_probe_xe(xf)
        u = rng.normal(size=24) * 1e-3
        el.update_probe_ue(u)
        KC0 = _coo(576)
        el.update_KC0(*KC0, prop, 0, *[float(v) for v in hg])
        KG = _coo(144)
        el.update_KG(*KG, prop)
        M0, M1, M2 = _coo(480), _coo(480), _coo(480)
        el.update_M(*M0, prop, mtype=0)
        el.update_M(*M1, prop, mtype=1)
        el.update_M(*M2, prop, mtype=2)
        fint = np.zeros(24)
        el.update_fint(fint, prop, *[float(v) for v in hg])
        finte = np.asarray(el.probe.finte).copy()
        Ns = rng.normal(size=3) * 1e3
        KGs = _coo(144)
        el.update_KG_given_stress(float(Ns[0]), float(Ns[1]), float(Ns[2]), *KGs)
        vals = dict(x=xf, c=c, xmat=xmat, pid=pid, u=u, k6rot=el.K6ROT, hg=hg,
                    R=[el.r11, el.r12, el.r13, el.r21, el.r22, el.r23, el.r31, el.r32, el.r33],
                    m=[el.m11, el.m12, el.m21, el.m22], xe=np.asarray(el.probe.xe).copy(),
                    area=el.area, ue=np.asarray(el.probe.ue).copy(),
                    KC0r=KC0[0], KC0c=KC0[1], KC0v=KC0[2], KGr=KG[0], KGc=KG[1], KGv=KG[2],
                    M0v=M0[2], M1v=M1[2], M2v=M2[2], fint=fint, finte=finte, Nstress=Ns,
                    KGsv=KGs[2])
        for k in keys:
            out[k].append(vals[k])
    return {k: np.array(v) for k, v in out.items()}


def tria3r_static():
    """The simply supported 7x11-node Tria3R plate with a unit centre load
    (the mesh of the reference's Tria3R static test)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.linalg import spsolve
    from pyfe3d import Tria3R, Tria3RData, Tria3RProbe, INT, DOUBLE, DOF
    from pyfe3d.shellprop_utils import isotropic_plate
    data = Tria3RData()
    probe = Tria3RProbe()
    nx, ny, a, b = 7, 11, 3., 7.
    xtmp = np.linspace(0, a, nx)
    ytmp = np.linspace(0, b, ny)
    xmesh, ymesh = np.meshgrid(xtmp, ytmp)
    ncoords = np.vstack((xmesh.T.flatten(), ymesh.T.flatten(), np.zeros(nx * ny))).T
    xf = ncoords.flatten()
    nids = np.arange(nx * ny).reshape(nx, ny)
    n1s = nids[:-1, :-1].flatten()
    n2s = nids[1:, :-1].flatten()
    n3s = nids[1:, 1:].flatten()
    n4s = nids[:-1, 1:].flatten()
    conn = []
    for n1, n2, n3, n4 in zip(n1s, n2s, n3s, n4s):
        conn.append((n1, n2, n3))
        conn.append((n1, n3, n4))
    conn = np.array(conn)
    E = len(conn)
    N = DOF * nx * ny
    KC0r = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=INT)
    KC0c = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=INT)
    KC0v = np.zeros(data.KC0_SPARSE_SIZE * E, dtype=DOUBLE)
    prop = isotropic_plate(thickness=0.005, E=200e9, nu=0.3, calc_scf=True)
    for e, (n1, n2, n3) in enumerate(conn):
        t = Tria3R(probe)
        t.c1, t.c2, t.c3 = DOF * n1, DOF * n2, DOF * n3
        t.alpha_shear_locking = 0.7
        t.init_k_KC0 = e * data.KC0_SPARSE_SIZE
        t.update_rotation_matrix(xf)
        t.update_probe_xe(xf)
        t.update_KC0(KC0r, KC0c, KC0v, prop)
    K = coo_matrix((KC0v, (KC0r, KC0c)), shape=(N, N)).tocsc()
    bk = np.zeros(N, dtype=bool)
    edge = (np.isclose(ncoords[:, 0], 0) | np.isclose(ncoords[:, 0], a) |
            np.isclose(ncoords[:, 1], 0) | np.isclose(ncoords[:, 1], b))
    for d in range(3):
        bk[d::DOF] = edge
    bu = ~bk
    f = np.zeros(N)
    middle = np.isclose(ncoords[:, 0], a / 2) & np.isclose(ncoords[:, 1], b / 2)
    f[2::DOF][middle] = 1.
    u = np.zeros(N)
    u[bu] = spsolve(K[bu, :][:, bu], f[bu])
    return dict(x=xf, conn=conn, bk=bk, f=f, u=u, prop=shell_rec(prop), Kdiag=K.diagonal(), nnz=K.nnz)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('PYFE3D_REF'),
                    help='path of the pyfe3d source tree (or set PYFE3D_REF)')
    args = ap.parse_args()
    if not args.ref:
        ap.error('give the pyfe3d source tree with --ref or PYFE3D_REF')
    import_reference(args.ref)
    rng = np.random.default_rng(20240611)
    names, recs, props = make_shell_props()
    inputs = []
    for name in names:
        inputs.append(name)
    np.savez_compressed(os.path.join(HERE, 'shellprop.npz'), names=np.array(names), records=recs)
    q = quad4_cases(props, rng)
    q['props'] = recs
    np.savez_compressed(os.path.join(HERE, 'quad4_elements.npz'), **q)
    b = beamc_cases(rng)
    np.savez_compressed(os.path.join(HERE, 'beamc_elements.npz'), **b)
    p = plate_static()
    np.savez_compressed(os.path.join(HERE, 'plate_static.npz'), **p)
    # the reduced-integration shells draw from their own streams, so the
    # fixtures above keep their values
    t = tria3r_cases(props, np.random.default_rng(33))
    t['props'] = recs
    np.savez_compressed(os.path.join(HERE, 'tria3r_elements.npz'), **t)
    q = quad4r_cases(props, np.random.default_rng(34))
    q['props'] = recs
    np.savez_compressed(os.path.join(HERE, 'quad4r_elements.npz'), **q)
    np.savez_compressed(os.path.join(HERE, 'tria3r_static.npz'), **tria3r_static())
    for f in ('shellprop', 'quad4_elements', 'beamc_elements', 'plate_static', 'tria3r_elements',
              'quad4r_elements', 'tria3r_static'):
        print(f, os.path.getsize(os.path.join(HERE, f + '.npz')), 'bytes')


if __name__ == '__main__':
    main()
