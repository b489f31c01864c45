"""Golden vectors of the reference's mode-to-ordinate binning (openbte/material.py RTA2DSym, RTA3D).

Test infrastructure only.  Runs the unmodified reference ``RTA2DSym`` (openbte/material.py:105-189) and
``RTA3D`` (openbte/material.py:7-102) through ``ref_loader`` on seeded synthetic mode data (no material
database is copied) and freezes inputs and outputs into ``material_rta.npz``.

Mode data: heat capacity U(0.2, 1) x 1e5 J/m^3/K, scattering time log-uniform in [1e-13, 1e-9] s, group
velocity a random direction times a speed U(200, 8000) m/s; a few modes have tau = 0 (zero MFP, removed by
the 1e-10 m filter) to exercise the filter.

Run: python tests/golden/make_golden_material.py   (needs the reference checkout)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))   # ref_loader
import ref_loader  # noqa: E402


def seeded_modes(n, seed):
    rng = np.random.default_rng(seed)
    cv = rng.uniform(0.2, 1.0, n) * 1e5
    tau = 10.0 ** rng.uniform(-13, -9, n)
    tau[:5] = 0.0
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    vg = d * rng.uniform(200.0, 8000.0, n)[:, None]
    return cv, tau, vg


def main():
    ref = ref_loader.load()
    out = {}
    cv, tau, vg = seeded_modes(1500, 11)
    out.update(cv=cv, tau=tau, vg=vg)
    data = ref.objects.MaterialRTA(cv.copy(), tau.copy(), vg.copy())
    for tag, kw in (("d2a", dict(n_phi=16, n_mfp=10)), ("d2b", dict(n_phi=48, n_mfp=30))):
        m = ref.material.RTA2DSym(data, **dict(kw))
        for f in ("thermal_conductivity", "sigma", "vmfp", "t_coeff", "mfps", "h", "heat_source_coeff"):
            out[f"{tag}_{f}"] = np.asarray(getattr(m, f), dtype=np.float64)
    for tag, kw in (("d3a", dict(n_phi=8, n_theta=6, n_mfp=8)),):
        m = ref.material.RTA3D(data, **dict(kw))
        for f in ("thermal_conductivity", "sigma", "vmfp", "t_coeff", "mfps", "h", "heat_source_coeff"):
            out[f"{tag}_{f}"] = np.asarray(getattr(m, f), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "material_rta.npz"), **out)
    print("wrote", os.path.join(HERE, "material_rta.npz"), sorted(out))


if __name__ == "__main__":
    main()
