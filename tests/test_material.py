"""Mode-to-ordinate binning (RTA2DSym, RTA3D) against the reference's own outputs, and the material loader."""
import os
import pickle
import sqlite3
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "material_rta.npz"))
FIELDS = ("thermal_conductivity", "sigma", "vmfp", "t_coeff", "mfps", "h", "heat_source_coeff")


def _data():
    from openbte_gb300.objects import MaterialRTA
    return MaterialRTA(GOLD["cv"], GOLD["tau"], GOLD["vg"])


def _check(m, tag):
    for f in FIELDS:
        want = GOLD[f"{tag}_{f}"]
        got = np.asarray(getattr(m, f), dtype=np.float64)
        assert got.shape == want.shape, (f, got.shape, want.shape)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * np.abs(want).max(), err_msg=f)


@pytest.mark.parametrize("tag,kw", [("d2a", dict(n_phi=16, n_mfp=10)), ("d2b", dict(n_phi=48, n_mfp=30))])
def test_rta2dsym_matches_reference(tag, kw):
    from openbte_gb300.material import RTA2DSym
    m = RTA2DSym(_data(), **kw)
    _check(m, tag)
    assert m.grid == (kw["n_mfp"], kw["n_phi"])
    assert abs(m.t_coeff.sum() - 1) < 1e-12


def test_rta3d_matches_reference():
    from openbte_gb300.material import RTA3D
    m = RTA3D(_data(), n_phi=8, n_theta=6, n_mfp=8)
    _check(m, "d3a")
    assert m.grid == (8, 6, 8)


def test_binning_conserves_mode_sums():
    """Bilinear weights sum to one per mode: the binned W and sigma keep the modes' totals."""
    from openbte_gb300.material import RTA2DSym
    d = _data()
    m = RTA2DSym(d, n_phi=24, n_mfp=12)
    tau = d.scattering_time
    keep = np.linalg.norm(d.group_velocity[:, :2] * tau[:, None], axis=1) > 1e-10
    W = (d.heat_capacity / np.where(tau > 0, tau, 1))[keep]
    sig = (d.heat_capacity[:, None] * d.group_velocity[:, :2])[keep]
    np.testing.assert_allclose(m.heat_source_coeff, 1 / W.sum(), rtol=1e-12)
    np.testing.assert_allclose(m.sigma.sum(axis=(0, 1)) * 1e9, sig.sum(axis=0), rtol=1e-9, atol=1e-9 * np.abs(sig).sum())


def test_load_rta_reads_sqlitedict_layout(tmp_path):
    from openbte_gb300.material import load_rta
    d = _data()
    fn = tmp_path / "Xx_rta.db"
    con = sqlite3.connect(fn)
    con.execute("CREATE TABLE unnamed (key TEXT PRIMARY KEY, value BLOB)")
    # rows in a different order than the fields: matched by name
    for k, v in (("group_velocity", d.group_velocity), ("heat_capacity", d.heat_capacity),
                 ("scattering_time", d.scattering_time), ("thermal_conductivity", np.eye(3))):
        con.execute("INSERT INTO unnamed VALUES (?, ?)", (k, pickle.dumps(v)))
    con.commit()
    con.close()
    m = load_rta("Xx_rta", path=str(tmp_path))
    np.testing.assert_array_equal(m.heat_capacity, d.heat_capacity)
    np.testing.assert_array_equal(m.group_velocity, d.group_velocity)
    np.testing.assert_array_equal(m.thermal_conductivity, np.eye(3))
    with pytest.raises(FileNotFoundError):
        load_rta("absent", path=str(tmp_path))


def test_real_silicon_against_reference():
    """Si_rta.db of the reference checkout, binned by both implementations (skipped without the checkout)."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import ref_loader
    if not ref_loader.available():
        pytest.skip("reference checkout not present")
    from openbte_gb300.material import RTA2DSym, load_rta
    folder = os.path.join(ref_loader.REF_ROOT, "openbte", "materials")
    if not os.path.isfile(os.path.join(folder, "Si_rta.db")):
        pytest.skip("Si_rta.db not present")
    ref = ref_loader.load()
    d = load_rta("Si_rta", path=folder)
    rd = ref.objects.MaterialRTA(d.heat_capacity.copy(), d.scattering_time.copy(), d.group_velocity.copy())
    want = ref.material.RTA2DSym(rd, n_phi=48, n_mfp=50)
    got = RTA2DSym(d, n_phi=48, n_mfp=50)
    for f in FIELDS:
        w = np.asarray(getattr(want, f), dtype=np.float64)
        np.testing.assert_allclose(np.asarray(getattr(got, f), dtype=np.float64), w, rtol=1e-10,
                                   atol=1e-10 * np.abs(w).max(), err_msg=f)
