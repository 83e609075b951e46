"""The C-ABI library loads and exports every entry point declared in
include/gbfusion.h; host-only entry points work without a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def L():
    from libfusion_gb300 import build as B
    B.build()
    import libfusion_gb300 as L
    return L


def declared():
    src = (ROOT / "include" / "gbfusion.h").read_text()
    return sorted(set(re.findall(r"GBF_API\s+[\w\s\*]+?\b(gbf_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(L):
    names = declared()
    assert len(names) >= 30
    lib = C.CDLL(str(L._lib.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert sorted(L._lib.SIGNATURES) == names


def test_version_and_defaults(L):
    assert "sm_103a" in L.version()
    c = L.default_config()
    # MapStruct defaults (src/data_struct/map_struct.cu:17-35)
    assert c.num_buckets == 200000 and c.num_blocks == 200000
    assert abs(c.voxel_size - 0.01) < 1e-9 and abs(c.truncation - 0.05) < 1e-7
    assert abs(c.zmax_update - 1.5) < 1e-7 and abs(c.zmin_update - 0.3) < 1e-7
    assert list(c.max_iterations)[:3] == [10, 5, 3]
    assert c.w_icp == 1e6 and c.w_rgb == 1.0
    assert c.motion_prior == 0  # each frame starts from no motion, as DenseOdometry::trackFrame does


def test_session_bytes_and_validation(L):
    K = L.IntrinsicMatrix(640, 480, 525, 525, 319.5, 239.5)
    c = L.default_config(num_blocks=1 << 17, num_buckets=1 << 18)
    n = L.session_bytes(c, K)
    assert n > (1 << 17) * 512 * 10  # voxel pool dominates (REF layout: 10 B / voxel)
    c.voxel_layout = L.VOXEL_HALF
    half = L.session_bytes(c, K)
    assert half < n
    c.voxel_layout = L.VOXEL_SNORM  # same 8 B per voxel as HALF
    assert L.session_bytes(c, K) == half
    for bad in (dict(num_levels=0), dict(num_levels=6), dict(voxel_size=0.0), dict(num_blocks=0),
                dict(voxel_layout=3), dict(voxel_layout=-1), dict(max_probe=0), dict(motion_prior=2)):
        cb = L.default_config(**bad)
        with pytest.raises(L.GbfError):
            L.session_bytes(cb, K)
    with pytest.raises(L.GbfError):
        L.session_bytes(L.default_config(), L.IntrinsicMatrix(642, 480, 525, 525, 320, 240))


def test_synthetic_poses_are_deterministic(L):
    import numpy as np
    a, b = L.SynthScene(seed=5), L.SynthScene(seed=5)
    for k in (0, 17, 199):
        Ta, Tb = a.pose(k), b.pose(k)
        assert np.array_equal(Ta, Tb)
        R = Ta[:3, :3]
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-12)
    fig8 = L.SynthScene(trajectory=1, room=(8, 8, 3), radius=2.5, speed=0.5, fps=30)
    step = np.linalg.norm(fig8.pose(1)[:3, 3] - fig8.pose(0)[:3, 3])
    assert abs(step - 0.5 / 30) < 2e-3


def test_session_create_without_gpu_fails_loudly(L):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    K = L.IntrinsicMatrix(160, 120, 131.25, 131.25, 79.875, 59.875)
    with pytest.raises(L.GbfError) as e:
        L.System(K, L.default_config())
    assert e.value.status in (2, 5)
