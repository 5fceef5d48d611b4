"""Restart files (FElib's scale_file_restart_meshfield.F90:136-186 content in a flat little-endian
file; layout in fe-project_gb300/csrc/fedg_restart.cu), host side: the numpy writer and reader
(fe-project_gb300/fedg/restart.py) round-trip every bit, and an oracle run split by a save and a
restore equals the uninterrupted run bit for bit."""
import numpy as np

import oracle as orc
from fedg import cases
from fedg import restart as rs


def test_numpy_round_trip_is_bit_exact(tmp_path):
    case = cases.C2().scaled(2, 2, 3)
    q, b = cases.initial_state(case)
    rng = np.random.default_rng(4)
    f = {nm: a + 1e-3 * rng.standard_normal(a.shape) for nm, a in zip(rs.NAMES[:5], q)}
    f.update(DENS_hyd=b["dens_hyd"], PRES_hyd=b["pres_hyd"], THERM_hyd=b["therm_hyd"])
    r = rs.Restart(case.porder, case.NeX, case.NeY, case.NeZ, step=123456789012, time=61.5, dt=0.04,
                   scheme="IMEX_ARK232", ref_wind=(10.25, -3.0), fields=f)
    p = tmp_path / "state.rst"
    rs.write(p, r)
    assert p.stat().st_size == rs.HEADER + 8 * len(rs.NAMES) * case.Ne * case.Np
    g = rs.read(p)
    assert (g.porder, g.NeX, g.NeY, g.NeZ, g.step, g.time, g.dt, g.scheme, g.ref_wind) == \
        (case.porder, case.NeX, case.NeY, case.NeZ, 123456789012, 61.5, 0.04, "IMEX_ARK232", (10.25, -3.0))
    for nm in rs.NAMES:
        assert np.array_equal(g.fields[nm].view(np.uint64), f[nm].view(np.uint64)), nm


def test_oracle_run_split_by_restart_is_bit_exact(tmp_path):
    """HEVI ARK232, Newton to 1e-12: 3 + 3 steps through a restart file == 6 steps."""
    case = cases.C1().scaled(3, 3, 3)
    q, b = cases.initial_state(case)
    o = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o.set_base_state(b["dens_hyd"], b["pres_hyd"])
    full, _, _ = o.step_hevi(q, 0.02, 6, max_iter=20, tol=1e-12)
    half, _, _ = o.step_hevi(q, 0.02, 3, max_iter=20, tol=1e-12)
    f = dict(zip(rs.NAMES[:5], half))
    f.update(DENS_hyd=b["dens_hyd"], PRES_hyd=b["pres_hyd"], THERM_hyd=b["therm_hyd"])
    rs.write(tmp_path / "s.rst", rs.Restart(case.porder, case.NeX, case.NeY, case.NeZ, 3, 0.06, 0.02, "IMEX_ARK232",
                                            None, f))
    r = rs.read(tmp_path / "s.rst")
    o2 = orc.Oracle(case.porder, case.NeX, case.NeY, case.NeZ, case.dom)
    o2.set_base_state(r.fields["DENS_hyd"], r.fields["PRES_hyd"])
    rest, _, _ = o2.step_hevi([r.fields[nm] for nm in rs.NAMES[:5]], 0.02, 3, max_iter=20, tol=1e-12)
    for v in range(5):
        assert np.array_equal(rest[v], full[v]), v
