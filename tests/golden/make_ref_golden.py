"""Generate tests/golden/ref_cases.npz: the outputs of nikikilbertus/InstaHeat's
own code (compiled unmodified by oracle/ref.py against the shims in
oracle/ref_shim/) for the cases in tests/ref_cases.py marked golden.

Run in a checkout whose reference sources are staged, e.g.
    python -c "from oracle import ref; ref.stage('/path/to/InstaHeat')"
    python tests/golden/make_ref_golden.py
The fixture is committed; tests fall back to it where the reference's
sources are not staged (a host without the reference checkout).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

import ref_cases  # noqa: E402


def main():
    from oracle import ref
    if not ref.available():
        raise SystemExit("stage the reference's sources first (oracle.ref.stage)")
    out = {}
    for name, case in ref_cases.CASES.items():
        if not case.get("golden"):
            continue
        r = ref_cases.run_reference(name)
        for k, v in r.items():
            out[f"{name}/{k}"] = np.asarray(v)
        print(name, {k: np.shape(v) for k, v in r.items()})
    np.savez_compressed(ref_cases.GOLDEN, **out)
    print("wrote", ref_cases.GOLDEN, ref_cases.GOLDEN.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
