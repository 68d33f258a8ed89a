import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "lsd-slam-pangolin-gui_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device (sm_103a)")


_cache = {}


def cached(key, fn):
    if key not in _cache:
        _cache[key] = fn()
    return _cache[key]


@pytest.fixture(scope="session")
def pair0():
    import synth
    return cached(("pair", 0, 640, 480), lambda: synth.tracking_pair(0))


@pytest.fixture(scope="session")
def pairs4():
    import synth
    return [cached(("pair", s, 640, 480), lambda s=s: synth.tracking_pair(s)) for s in range(4)]


@pytest.fixture(scope="session")
def small_pair():
    import synth
    return cached(("pair", 7, 160, 128), lambda: synth.tracking_pair(7, 160, 128))


@pytest.fixture(scope="session")
def ctx():
    import lsdg
    c = lsdg.Context()
    yield c
    c.close()
