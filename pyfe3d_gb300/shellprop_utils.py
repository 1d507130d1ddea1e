"""Laminate builders with the signatures of ``pyfe3d.shellprop_utils``
(pyfe3d/shellprop_utils.py:13-206)."""
from .shellprop import Lamina, MatLamina, ShellProp


def read_laminaprop(laminaprop, rho=0):
    """MatLamina from a 2-, 6- or 9-tuple (shellprop_utils.py:13-93)."""
    matlam = MatLamina()
    assert len(laminaprop) in (2, 6, 9), ('Invalid entry for laminaprop: ' + str(laminaprop))
    if len(laminaprop) == 2:
        e, nu = laminaprop
        g = e / (2 * (1 + nu))
        laminaprop = (e, e, nu, g, g, g, 0, 0, 0)
    elif len(laminaprop) == 6:
        laminaprop = tuple(list(laminaprop) + [0, 0, 0])
    matlam.e1 = laminaprop[0]
    matlam.e2 = laminaprop[1]
    matlam.e3 = laminaprop[6]
    matlam.nu12 = laminaprop[2]
    matlam.nu13 = laminaprop[7]
    matlam.nu23 = laminaprop[8]
    matlam.nu21 = matlam.nu12 * matlam.e2 / matlam.e1
    matlam.nu31 = matlam.nu13 * matlam.e3 / matlam.e1
    matlam.nu32 = matlam.nu23 * matlam.e3 / matlam.e2
    matlam.g12 = laminaprop[3]
    matlam.g13 = laminaprop[4]
    matlam.g23 = laminaprop[5]
    matlam.rho = rho
    matlam.rebuild()
    return matlam


def laminated_plate(stack, plyt=None, laminaprop=None, rho=0., plyts=None, laminaprops=None,
                    rhos=None, offset=0., calc_scf=True):
    """ShellProp of a stacking sequence (shellprop_utils.py:96-179)."""
    prop = ShellProp()
    prop.offset = offset
    prop.stack = list(stack)
    if plyts is None:
        if plyt is None:
            raise ValueError('plyt or plyts must be supplied')
        plyts = [plyt for _ in stack]
    if laminaprops is None:
        if laminaprop is None:
            raise ValueError('laminaprop or laminaprops must be supplied')
        laminaprops = [laminaprop for _ in stack]
    if rhos is None:
        rhos = [rho for _ in stack]
    if not (len(stack) == len(plyts) == len(laminaprops) == len(rhos)):
        raise ValueError('stack, plyts, laminaprops and rhos must have the same length')
    plies = []
    prop.h = 0.
    for t, lp, thetadeg, r in zip(plyts, laminaprops, stack, rhos):
        ply = Lamina()
        ply.thetadeg = float(thetadeg)
        ply.h = t
        prop.h += ply.h
        ply.matlamina = read_laminaprop(lp, r)
        ply.rebuild()
        plies.append(ply)
    prop.plies = plies
    prop.calc_constitutive_matrix()
    prop.calc_equivalent_properties()
    if calc_scf:
        prop.calc_scf()
    return prop


def isotropic_plate(thickness, E, nu, offset=0., calc_scf=True, rho=0.):
    """Single 0-degree ply of an isotropic material (shellprop_utils.py:182-206)."""
    return laminated_plate(plyt=thickness, stack=[0], laminaprop=(E, nu), rho=rho, offset=offset,
                           calc_scf=calc_scf)
