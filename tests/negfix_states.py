"""Moist states for the tracer negative fixer's tests: a base state of the flat cube with six water
species (vapour, two liquid, three ice: QLA = 2, QIA = 3), some of them negative in places, and the
element geometry the fixer integrates with (the LGL quadrature weights times the volume Jacobian,
the node heights)."""
import numpy as np

from fedg import cases
from fedg.element import lgl_nodes

QLA, QIA = 2, 3
# representative tracer properties (scale_tracer's TRACER_MASS, _R, _CV, _CP) of water vapour,
# liquid and ice [J/kg/K]
MASS = [1.0] * 6
R = [461.46, 0.0, 0.0, 0.0, 0.0, 0.0]
CV = [1384.14, 4218.0, 4218.0, 2106.0, 2106.0, 2106.0]
CP = [1845.60, 4218.0, 4218.0, 2106.0, 2106.0, 2106.0]


def geometry(case):
    """(int_w (Np,), zlev (Ne, Np)) of the flat cube: J w_i w_j w_k and the node heights"""
    _, w = lgl_nodes(case.porder)
    xmin, xmax, ymin, ymax, zmin, zmax = case.dom
    jac = (xmax - xmin) / case.NeX * (ymax - ymin) / case.NeY * (zmax - zmin) / case.NeZ / 8.0
    wk, wj, wi = np.meshgrid(w, w, w, indexing="ij")
    int_w = (jac * wi * wj * wk).reshape(-1)
    _, _, z = cases.node_coords(case)
    return int_w, z


def moist_state(case, seed=0, neg_frac=0.2, neg_elems=()):
    """(qtrc (6, Ne, Np), ddens, pres, cvtot, cptot, rtot, dens_hyd, pres_hyd, drhot) with Rtot, CVtot,
    CPtot those of the mixing ratios and PRES that of DRHOT with the mixture's exponent.  A fraction
    neg_frac of the condensate values is negative (small undershoots of a transport step); in the
    elements neg_elems the first condensate is negative throughout (a negative element mass)."""
    from negfix_ref import specific_heat

    rng = np.random.default_rng(seed)
    q0, b = cases.initial_state(case)
    dens_hyd, pres_hyd = b["dens_hyd"], b["pres_hyd"]
    ddens = q0[0] + 1e-4 * rng.standard_normal(dens_hyd.shape)
    qv = 1e-2 * (0.5 + 0.5 * rng.random(dens_hyd.shape))
    qc = [1e-4 * rng.random(dens_hyd.shape) for _ in range(5)]
    for a in qc:
        neg = rng.random(a.shape) < neg_frac
        a[neg] = -1e-6 * rng.random(int(neg.sum()))
    for e in neg_elems:
        qc[0][e] = -1e-6 * (0.5 + rng.random(case.Np))
    qtrc = np.stack([qv] + qc)
    _, rtot, cvtot, cptot = specific_heat(qtrc, MASS, R, CV, CP, cases.RDRY, cases.CVDRY, cases.CPDRY)
    rhot_hyd = cases.PRES00 / cases.RDRY * (pres_hyd / cases.PRES00) ** (cases.CVDRY / cases.CPDRY)
    drhot = q0[4]
    pres = cases.PRES00 * (rtot * (rhot_hyd + drhot) / cases.PRES00) ** (cptot / cvtot)
    return qtrc, ddens, pres, cvtot, cptot, rtot, dens_hyd, pres_hyd, drhot
