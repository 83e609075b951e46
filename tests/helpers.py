"""Shared helpers for the tests: small configurations and synthetic frames."""
import numpy as np


def small_config(L, layout=0, **over):
    kw = dict(voxel_size=0.01, truncation=0.03, zmin_update=0.3, zmax_update=4.0, zmin_raycast=0.3,
              zmax_raycast=4.0, num_buckets=1 << 17, num_blocks=1 << 15, voxel_layout=layout, num_levels=3,
              max_iterations=[10, 5, 3, 3, 3], bilateral=1, max_probe=128)
    kw.update(over)
    return L.default_config(**kw)


def intrinsics(L, w=320, h=240):
    s = w / 640.0
    return L.IntrinsicMatrix(w, h, 525.0 * s, 525.0 * s, 319.5 * s, 239.5 * s)


def frames(L, K, n, start=0, step=1, **scene):
    """n synthetic frames (depth u16 mm, rgb8, ground-truth pose) as numpy."""
    import torch
    sc = L.SynthScene(**scene)
    out = []
    for i in range(n):
        k = start + i * step
        d, c = sc.render(K, k)
        torch.cuda.synchronize()
        out.append((d.cpu().numpy(), c.cpu().numpy(), sc.pose(k)))
    return out


def depth_m(d_u16):
    return d_u16.astype(np.float32) * np.float32(0.001)


def cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def sort_blocks(coords, *arrays):
    order = np.lexsort((coords[:, 2], coords[:, 1], coords[:, 0]))
    return (coords[order],) + tuple(a[order] for a in arrays)


def sort_tris(v, *attrs):
    """Canonical triangle order: by the 9 vertex coordinates, ties broken by
    the attributes (duplicate triangles from neighbouring cubes)."""
    cols = [v.reshape(len(v), 9)[:, i] for i in range(9)]
    for a in attrs:
        flat = a.reshape(len(a), -1).astype(np.float64)
        cols += [np.nan_to_num(flat[:, i], nan=1e30) for i in range(flat.shape[1])]
    order = np.lexsort(cols[::-1])
    return (v[order],) + tuple(a[order] for a in attrs)
