"""Generate tests/golden/flrw_homogeneous.json by importing the reference's own
homogeneous-FLRW helper (nikikilbertus/InstaHeat helpers/flrw_homogeneous.py,
which integrates phi'' = -3 H phi' - V', H = sqrt((phi'^2/2 + V)/3), a' = H a
with scipy's dopri5 at rtol 1e-8, atol 1e-10).

Run in a container that has the reference checked out:
    python tests/golden/make_flrw_golden.py /path/to/InstaHeat
The helper imports matplotlib only for plotting in its __main__ block, so a
stub module stands in for it.  The JSON is committed; tests never read the
reference at run time.
"""
import importlib.util
import json
import sys
import types
from pathlib import Path

import numpy as np


def load_helper(ref_root: Path):
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
    spec = importlib.util.spec_from_file_location(
        "flrw_homogeneous", ref_root / "helpers" / "flrw_homogeneous.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_flrw_golden.py /path/to/InstaHeat")
    ref_root = Path(sys.argv[1])
    mod = load_helper(ref_root)
    cases = []
    for phi0 in (1.0, 0.8, 1.2):
        V = 0.5 * phi0 ** 2
        dphi0 = -phi0 / (3.0 * np.sqrt(V / 3.0))  # slow roll, m = 1
        u = mod.inflation(phi0, dphi0)
        t, phi, phi_dot, a, H = u.integrate(10.0, 20)
        cases.append({"phi0": phi0, "dphi0": dphi0, "t": t.tolist(), "phi": phi.tolist(),
                      "phi_dot": phi_dot.tolist(), "a": a.tolist(), "H": H.tolist()})
    out = Path(__file__).with_name("flrw_homogeneous.json")
    out.write_text(json.dumps({"source": "helpers/flrw_homogeneous.py (scipy dopri5, rtol 1e-8, atol 1e-10)",
                               "mass": 1.0, "cases": cases}, indent=1))
    print("wrote", out)


if __name__ == "__main__":
    main()
