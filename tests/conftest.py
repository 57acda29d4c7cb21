"""Shared pytest setup: markers, import paths, and small-grid fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "bacterial-droplet_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__)),
          os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def random_state(N, seed, amp=0.05):
    """A smooth droplet plus small random u, P, u*, P* (every field non-zero)."""
    import ttsh
    rng = np.random.default_rng(seed)
    phi, P = ttsh.init_droplet(N, R=N / 4, xi=2.0, seed=seed)
    noise = lambda: amp * rng.standard_normal((3, N, N, N))
    P = P + 0.5 * noise()
    return dict(phi=phi, P=P, u=noise(), us=noise(), ps=noise())


def oracle_state(st):
    """dict for oracle.step from a random_state dict."""
    import oracle as O
    N = st["phi"].shape[0]
    s = O.new_state(N)
    s["phi"][:] = st["phi"]
    for b, c in enumerate("xyz"):
        s["p" + c][:] = st["P"][b]
        s["v" + c][:] = st["u"][b]
        s["v" + c + "s"][:] = st["us"][b]
        s["p" + c + "s"][:] = st["ps"][b]
    return s


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build()
    return O
