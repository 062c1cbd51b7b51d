"""Shared fixtures: the `gpu` marker, seeded scenes, and the built libraries."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build as ob
    ob.build_oracle()
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def product_lib():
    from voxelhashmt_gb300 import build as pb
    pb.build()
    from voxelhashmt_gb300 import _capi
    _capi.lib()
    return _capi


@pytest.fixture(scope="session")
def small_orbit():
    """Config-1 geometry at 64x48 (focal length scaled with the resolution), 24 orbit poses, with the
    reference volume's default voxel size and truncation (voxel_hash_tsdf.h:191-192: 2 cm, 6 cm) so the
    oracle finishes in about a second."""
    from voxelhashmt_gb300 import scenes
    sc = scenes.orbit_scene(seed=7, frames=24, width=64, height=48, fx=277.0 * 0.2, fy=277.0 * 0.2,
                            cx=32.0, cy=24.0)
    sc.voxel_size, sc.truncation = 0.02, 0.06
    return sc
