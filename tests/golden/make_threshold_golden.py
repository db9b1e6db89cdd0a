#!/usr/bin/env python3
"""Generate the setThreshold (src/isolevel.c:245-277) fixtures from the
reference nii2mesh itself: edge cases of the robust range and of the Otsu
searches that the meshing fixtures do not reach.

Run where the reference tree exists (it builds oracle/_ref from the
reference's own sources):  python tests/golden/make_threshold_golden.py

Writes
  threshold_inputs.npz   the seeded input arrays (stored, so every machine
                         thresholds bit-identical inputs)
  threshold.json         {case: {mode: value}} from the reference, modes 1-3
"""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from nii2mesh_gb300 import synth  # noqa: E402
from oracle.oracle import Reference  # noqa: E402

from oracle.refpath import reference_src  # noqa: E402

SRC = reference_src()   # N2M_REFERENCE, or a `reference` checkout beside this repository


def cases():
    rng = np.random.default_rng(77)
    c = {}
    c["constant"] = np.full(5000, 42.0, np.float32)                       # no variability
    c["all_nan"] = np.full(3000, np.nan, np.float32)                      # nothing but NaN
    c["tiny"] = rng.normal(10, 3, 60).astype(np.float32)                  # < 100 voxels: full range
    v = rng.normal(0, 1, 20000).astype(np.float32)
    v[rng.random(20000) < 0.1] = np.nan
    c["with_nan"] = v                                                     # NaNs skipped everywhere
    v = np.zeros(40000, np.float32)
    v[:9000] = rng.gamma(3.0, 40.0, 9000)
    c["zero_background"] = v                                              # MRI-like: mostly zeros
    c["negative"] = (-500.0 - rng.gamma(2.0, 100.0, 30000)).astype(np.float32)
    v = rng.integers(0, 256, 50000).astype(np.float32)
    v[rng.random(50000) < 0.6] = 0.0
    c["u8_ties"] = v                                                      # integer data, many ties
    c["binary"] = (rng.random(30000) < 0.3).astype(np.float32)            # robust range of a mask
    c["bimodal"] = np.concatenate([rng.normal(20, 5, 15000), rng.normal(200, 30, 5000)]).astype(np.float32)
    c["trimodal"] = np.concatenate([rng.normal(0, 4, 9000), rng.normal(60, 6, 9000),
                                    rng.normal(150, 10, 9000)]).astype(np.float32)
    c["heavy_tail"] = rng.standard_cauchy(40000).astype(np.float32)       # 2 %/98 % cut the tails
    c["outlier"] = np.concatenate([rng.normal(100, 10, 30000), [1e6]]).astype(np.float32)
    c["ct_slab"] = synth.ct512(seed=9, n=40, count=4).ravel()
    c["brain_third"] = synth.brain()[::3, ::3, ::3].astype(np.float32).ravel()
    return c


def main():
    subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh"), str(SRC)], check=True, stdout=subprocess.DEVNULL)
    ins = cases()
    np.savez_compressed(HERE / "threshold_inputs.npz", **ins)
    ref = Reference(False)
    out = {name: {str(m): ref.set_threshold(a, m) for m in (1, 2, 3)} for name, a in ins.items()}
    (HERE / "threshold.json").write_text(json.dumps(out, indent=1, sort_keys=True))
    print(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
