"""The GPU snapshot reductions (centroid, centroid slice, vorticities) against the numpy
restatement of readDraw.py / op.py: FP64 fields to 1e-12 (the vorticity is a 5-point sum)."""
import numpy as np
import pytest

import readdraw_restatement as RD
from conftest import random_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [64, 32])
def test_snapshot_slice_matches_readdraw(precision):
    import ttsh
    N = 32
    st = random_state(N, seed=5)
    # move the droplet off-centre so that the centroid is not near an integer
    st["phi"] = np.roll(st["phi"], (3, -2, 5), axis=(0, 1, 2)) * 0.9 + 0.01
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    with ttsh.Sim(inp, ttsh.default_ext(precision=precision)) as s:
        s.set_state(0, st["phi"], st["P"], st["u"])
        g = s.get_state(0)
        got = s.snapshot_slice(0)
    want = RD.analyse(g["phi"], g["P"], g["u"])
    assert got["index"] == want["index"]
    np.testing.assert_allclose(got["centroid"], want["centroid"], rtol=1e-12)
    for k in ttsh.Sim.SLICE_NAMES:
        np.testing.assert_allclose(got[k], want[k], rtol=0, atol=1e-12 * max(1.0, np.abs(want[k]).max()), err_msg=k)
