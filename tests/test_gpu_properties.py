"""Property sweeps on the GPU (seeded, so they run where hypothesis is not
installed): the block table under adversarial collisions -- every block of a
set that shares one home slot is stored, found and collected; past the probe
limit the overflow is refused and reported -- and block collection against
numpy's selection for keep masks from empty to full."""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

CAP = 1 << 12  # hash slots (a power of two: the home slot is the hash's low bits)


def _home_slot(c):
    """computeHash (map_struct.cu:143-148) modulo a power-of-two slot count, in
    32-bit unsigned arithmetic as the table computes it."""
    c = np.asarray(c, np.int64)
    ux = (c[:, 0].astype(np.uint32) * np.uint32(73856093))
    uy = (c[:, 1].astype(np.uint32) * np.uint32(19349669))
    uz = (c[:, 2].astype(np.uint32) * np.uint32(83492791))
    return ((ux ^ uy ^ uz) & np.uint32(CAP - 1)).astype(np.int64)


def _colliding(n, seed=0):
    """n distinct block coordinates that all hash to the same home slot."""
    rng = np.random.default_rng(seed)
    with np.errstate(over="ignore"):
        c = rng.integers(-4000, 4000, size=(4_000_000, 3), dtype=np.int64)
        s = _home_slot(c)
    target = np.bincount(s).argmax()
    pick = np.unique(c[s == target], axis=0)
    assert len(pick) >= n
    return pick[rng.permutation(len(pick))[:n]].astype(np.int32), int(target)


def _blocks(coords, seed):
    rng = np.random.default_rng(seed)
    n = len(coords)
    sdf = np.zeros((n, 512), np.float32)  # 0 and 1 are stored exactly in every layout
    w = np.ones((n, 512), np.float32)
    rgb = rng.integers(0, 256, size=(n, 512, 3), dtype=np.uint8)
    return coords, sdf, w, rgb


@pytest.mark.parametrize("layout", [0, 2])
def test_colliding_blocks_are_stored_found_and_collected(gbf, layout):
    L = gbf
    K = H.intrinsics(L)
    n = 300
    coords, slot = _colliding(n, seed=layout)
    with np.errstate(over="ignore"):
        assert np.all(_home_slot(coords) == slot)
    m = L.DenseMapping(K, H.small_config(L, layout, num_buckets=CAP, num_blocks=CAP, max_probe=512))
    m.import_blocks(*_blocks(coords, 1))
    assert m.stats().status == 0 and m.stats().allocated_blocks == n
    got = H.sort_blocks(*m.export())
    for x, y in zip(got, H.sort_blocks(*_blocks(coords, 1))):
        assert np.array_equal(x, y)
    # every other one out: the probe chain gets holes, the table is rebuilt
    # from the rest, each of which is still found
    gone, kept = coords[::2], coords[1::2]
    assert m.delete_blocks(gone) == len(gone)
    assert m.delete_blocks(gone) == 0
    assert {tuple(x) for x in m.export()[0]} == {tuple(x) for x in kept}
    assert m.delete_blocks(kept) == len(kept) and m.stats().allocated_blocks == 0


def test_collisions_past_the_probe_limit_are_refused_and_reported(gbf):
    L = gbf
    K = H.intrinsics(L)
    n, probe = 200, 64
    coords, _ = _colliding(n, seed=5)
    m = L.DenseMapping(K, H.small_config(L, 2, num_buckets=CAP, num_blocks=CAP, max_probe=probe))
    m.import_blocks(*_blocks(coords, 2))
    st = m.stats()
    assert st.status & L.FLAG_HASH_FULL
    # the first `probe` slots of the chain hold blocks, the rest were refused
    assert st.allocated_blocks == probe
    held = m.export()[0]
    assert len({tuple(x) for x in held} - {tuple(x) for x in coords}) == 0


MASKS = ["none", "all", "first", "last", "sparse", "dense", "alternate"]


@pytest.mark.parametrize("mask", MASKS)
def test_collection_matches_numpy_selection(gbf, mask):
    """Fused blocks collected with a keep mask of each kind: the map holds
    exactly numpy's selection, voxels unchanged, and every kept block is found."""
    L = gbf
    K = H.intrinsics(L)
    m = L.DenseMapping(K, H.small_config(L, 2))
    for d, c, T in H.frames(L, K, 3, step=3):
        m.update(H.cuda(H.depth_m(d)), H.cuda(c), T)
    c0, s0, w0, r0 = m.export()
    n = len(c0)
    assert n > 200
    rng = np.random.default_rng(MASKS.index(mask))
    gone = {"none": np.zeros(n, bool), "all": np.ones(n, bool),
            "first": np.arange(n) == 0, "last": np.arange(n) == n - 1,
            "sparse": rng.random(n) < 0.1, "dense": rng.random(n) < 0.9,
            "alternate": np.arange(n) % 2 == 0}[mask]
    assert m.delete_blocks(c0[gone]) == int(gone.sum())
    assert m.stats().allocated_blocks == int((~gone).sum())
    keep = ~gone
    for x, y in zip(H.sort_blocks(*m.export()), H.sort_blocks(c0[keep], s0[keep], w0[keep], r0[keep])):
        assert np.array_equal(x, y)
    assert m.delete_blocks(c0[keep]) == int(keep.sum())
