"""setThreshold (src/isolevel.c:245-277) on the GPU against the reference's
own values (tests/golden) and the oracle, bit for bit."""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
TH = json.loads((GOLD / "threshold.json").read_text())
TH_INPUTS = dict(np.load(GOLD / "threshold_inputs.npz"))
G = json.loads((GOLD / "golden.json").read_text())
INPUTS = dict(np.load(GOLD / "inputs.npz"))


@pytest.mark.parametrize("case", sorted(TH))
def test_threshold_edge_cases_dropin(gpu, case):
    for mode, val in TH[case].items():
        assert gpu.set_threshold(TH_INPUTS[case], int(mode)) == val, (case, mode)


def test_threshold_meshing_inputs(gpu):
    ctx = gpu.Context(0)
    for key, val in G["threshold"].items():
        name, mode = key.split(":")
        assert ctx.set_threshold(INPUTS[name], int(mode)) == val, key


def test_threshold_device_matches_oracle(gpu, oracle):
    """device-resident input, larger volumes (CT-like 96^3, brain-sized u8)"""
    import torch
    from nii2mesh_gb300 import synth
    ctx = gpu.Context(0)
    for vol in (synth.ct512(seed=4, n=96, count=12), synth.brain().astype(np.float32)):
        d = torch.from_numpy(np.ascontiguousarray(vol)).cuda()
        torch.cuda.synchronize()
        for mode in (1, 2, 3):
            assert ctx.set_threshold_device(d.data_ptr(), vol.size, mode) == oracle.set_threshold(vol, mode), mode


def test_threshold_empty_and_bad_args(gpu):
    import ctypes as C
    L = gpu.lib()
    out = C.c_float(0.0)
    ctx = gpu.Context(0)
    assert L.n2m_set_threshold(ctx.h, None, 0, 2, C.byref(out)) == 0 and out.value == 1.0   # no voxels: 1
    assert L.n2m_set_threshold(ctx.h, None, 10, 2, C.byref(out)) != 0                       # null volume
