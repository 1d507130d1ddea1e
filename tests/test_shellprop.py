"""Host ShellProp builders against the reference's frozen records (no GPU)."""
import numpy as np
import pytest

from pyfe3d_gb300.shellprop import isotropic_plate_records, shell_record
from pyfe3d_gb300.shellprop_utils import isotropic_plate, laminated_plate

LAM = (142.5e9, 8.7e9, 0.28, 5.1e9, 5.1e9, 5.1e9)
SPECS = {
    'iso_thin': lambda: isotropic_plate(0.005, 70e9, 0.33),
    'iso_rho': lambda: isotropic_plate(0.01, 70e9, 0.3, rho=2700),
    'iso_thick': lambda: isotropic_plate(0.8, 70e9, 0.3, rho=2700),
    'iso_offset': lambda: isotropic_plate(0.004, 200e9, 0.3, offset=0.001, rho=7800),
    'lam_quasi': lambda: laminated_plate([0, 45, -45, 90, 90, -45, 45, 0], plyt=0.000125,
                                         laminaprop=LAM),
    'lam_unsym': lambda: laminated_plate([0, 45, -45, 90, 30], plyt=0.0011, laminaprop=LAM,
                                         rho=1600, offset=0.001),
    'lam_iso2': lambda: laminated_plate([0, 90], plyt=0.002, laminaprop=(70e9, 0.33), rho=2700),
    'lam_noscf': lambda: laminated_plate([15, -15], plyt=0.001, laminaprop=LAM, calc_scf=False),
}


def test_records_match_reference(golden):
    g = golden('shellprop')
    for name, ref in zip(g['names'], g['records']):
        rec = shell_record(SPECS[str(name)]())
        scale = np.maximum(np.abs(ref), 1e-300)
        err = np.abs(rec - ref) / scale
        err[np.abs(ref) < 1e-30] = np.abs(rec - ref)[np.abs(ref) < 1e-30]
        assert err.max() < 1e-13, (name, err)


def test_vectorised_isotropic_records():
    h = np.array([0.001, 0.005, 0.02, 0.8])
    recs = isotropic_plate_records(h, 70e9, 0.33, rho=2700.)
    for i, hi in enumerate(h):
        ref = shell_record(isotropic_plate(hi, 70e9, 0.33, rho=2700.))
        np.testing.assert_allclose(recs[i], ref, rtol=1e-14, atol=0)


def test_laminate_properties_accessors():
    p = SPECS['lam_quasi']()
    assert p.ABD.shape == (6, 6) and p.ABDE.shape == (8, 8)
    assert np.allclose(p.B, 0, atol=1e-9 * np.abs(p.A).max())
    assert abs(p.h - 0.001) < 1e-15


@pytest.mark.gpu
def test_isotropic_records_on_device_match_host(gpulib):
    from pyfe3d_gb300.shellprop import isotropic_plate_records, isotropic_plate_records_device
    rng = np.random.default_rng(8)
    n = 5000
    h = 0.005 * np.exp(0.3 * rng.standard_normal(n))
    E = rng.uniform(50e9, 210e9, n)
    nu = rng.uniform(0.25, 0.35, n)
    rho = rng.uniform(1000., 8000., n)
    off = rng.uniform(-0.001, 0.001, n)
    for scf in (True, False):
        ref = isotropic_plate_records(h, E, nu, rho, off, calc_scf=scf)
        got = isotropic_plate_records_device(h, E, nu, rho, off, calc_scf=scf).cpu().numpy()
        err = np.abs(got - ref).max(axis=0) / np.maximum(np.abs(ref).max(axis=0), 1e-300)
        assert err.max() < 1e-13, err
    # scalars broadcast
    ref = isotropic_plate_records(h, 70e9, 0.33)
    got = isotropic_plate_records_device(h, 70e9, 0.33).cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.gpu
def test_laminate_records_on_device_match_reference_and_host(gpulib, golden):
    """Laminated records built on the device: the reference's frozen records of
    every builder case, and per-record stacks (thickness, angles, offsets,
    densities varying by record) against the host builder."""
    from pyfe3d_gb300.shellprop import laminate_records_device
    g = golden('shellprop')
    specs = {
        'iso_thin': ([0], 0.005, (70e9, 0.33), 0., 0., True),
        'iso_rho': ([0], 0.01, (70e9, 0.3), 2700., 0., True),
        'iso_thick': ([0], 0.8, (70e9, 0.3), 2700., 0., True),
        'iso_offset': ([0], 0.004, (200e9, 0.3), 7800., 0.001, True),
        'lam_quasi': ([0, 45, -45, 90, 90, -45, 45, 0], 0.000125, LAM, 0., 0., True),
        'lam_unsym': ([0, 45, -45, 90, 30], 0.0011, LAM, 1600., 0.001, True),
        'lam_iso2': ([0, 90], 0.002, (70e9, 0.33), 2700., 0., True),
        'lam_noscf': ([15, -15], 0.001, LAM, 0., 0., False),
    }
    for name, ref in zip(g['names'], g['records']):
        st, t, lp, rho, off, scf = specs[str(name)]
        got = laminate_records_device(st, t, lp, rho=rho, offset=off, calc_scf=scf).cpu().numpy()[0]
        _same_record(got, ref, name)
    rng = np.random.default_rng(12)
    n, nply = 300, 6
    th = rng.choice([0., 30., 45., -45., 60., 90.], size=(n, nply))
    pt = rng.uniform(1e-4, 5e-4, size=(n, nply))
    rho = rng.uniform(1000., 2000., size=(n, nply))
    off = rng.uniform(-2e-4, 2e-4, n)
    got = laminate_records_device(th, pt, LAM, rho=rho, offset=off).cpu().numpy()
    for i in range(0, n, 7):
        ref = shell_record(laminated_plate(th[i], plyts=list(pt[i]), laminaprop=LAM, rhos=list(rho[i]),
                                           offset=off[i]))
        _same_record(got[i], ref, i)


def _same_record(got, ref, what):
    """ABD and E to 1e-13 of their natural scales (|A|, |A| h, |A| h^2, |E|:
    entries that cancel, such as A16 of a balanced laminate or B of a
    symmetric one, carry only rounding noise), scf and h to 1e-13 relative."""
    h = ref[23]
    a = np.abs(ref[0:6]).max()
    for (lo, hi), scale in (((0, 6), a), ((6, 12), a * h), ((12, 18), a * h * h),
                            ((18, 21), np.abs(ref[18:21]).max())):
        assert np.abs(got[lo:hi] - ref[lo:hi]).max() <= 1e-13 * scale, (what, lo)
    assert np.allclose(got[21:24], ref[21:24], rtol=1e-13, atol=0), what
    # density integrals: int rho, int rho z (zero but for rounding on a
    # symmetric stack), int rho z^2, each to 1e-13 of int rho h^k
    for k in range(3):
        assert abs(got[24 + k] - ref[24 + k]) <= 1e-13 * abs(ref[24]) * h ** k, (what, 24 + k)
