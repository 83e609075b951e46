"""Generate tests/golden/ref_kernels.npz: outputs of the reference's own
integration, z-range / raycast, ICP-row and photometric-row kernels, run on a
GPU on the cases of tests/golden/pin_cases.py.

Needs a CUDA GPU, the oracle (oracle/, built by its Makefile), libgbfusion
(its synthetic renderer draws the two input frames; its host-only map-dump
writer lays the map out as the reference's chained hash table) and the
device modules oracle/_ref/pin_*.cubin, which oracle/ref_pin/build_kernels.sh
compiles from the reference sources where they lie.  The modules are built
where the reference tree is and carried to the GPU machine with the working
tree; this script runs there.  It prints, per case, whether the oracle on the
same machine matches, and writes the fixture (default
tests/golden/ref_kernels.npz).

It also stores CUDA's sinf of every argument the oracle's normal-weighted
update evaluates on these frames (sin_x, sin_y), recorded from the oracle and
evaluated on the GPU, so that the pin test can compare that update bit for bit.

Usage: python tests/golden/make_kernel_golden.py [OUT.npz]
"""
from __future__ import annotations

import ctypes as C
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "oracle", ROOT / "oracle" / "ref_pin", ROOT / "tests" / "golden"):
    sys.path.insert(0, str(p))

import pin_cases as P  # noqa: E402

REF = ROOT / "oracle" / "_ref"
REF_BLOCKS = 100000  # num_max_rendering_blocks_, the MapStruct default (map_struct.cu:27)
# RenderingBlock (include/data_struct/map_struct.h:62-67): Vector2s upper_left, lower_right; Vector2f zrange
SENTINEL = 12345.0  # what a pixel the image kernels do not write keeps
RENDERING_BLOCK = np.dtype([("upper_left", "<i2", 2), ("lower_right", "<i2", 2), ("zrange", "<f4", 2)])


def ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class Reference:
    """The pin modules of one build (-fmad=false, or nvcc's default contraction)."""

    def __init__(self, suffix: str = ""):
        import cudrv
        self.cu = cudrv
        self.m = {k: cudrv.Module(REF / f"pin_{k}{suffix}.cubin")
                  for k in ("fusion", "raycast", "icp", "rgb", "imgproc", "mesh")}
        import torch
        sz = torch.zeros(4, dtype=torch.int32, device="cuda")
        self.m["fusion"].function("pin_sizes").launch((1,), (1,), [ptr(sz)])
        # Voxel, HashEntry, RenderingBlock, MapState as the reference's headers lay them out
        assert sz.cpu().tolist() == [12, 20, 16, 40], sz.cpu().tolist()

    def set_state(self, mod: str, n_buckets: int, n_entries: int, n_blocks: int, max_triangles: int = 0):
        f = C.c_float
        self.m[mod].function("pin_set_state").launch(
            (1,), (1,), [C.c_int(n_buckets), C.c_int(n_entries), C.c_int(n_blocks), f(P.VOXEL), f(P.ZMIN), f(P.ZMAX),
                         f(P.ZMIN), f(P.ZMAX), C.c_int(REF_BLOCKS), C.c_int(max_triangles)])

    def state_values(self, mod: str):
        import torch
        out = torch.zeros(4, dtype=torch.float32, device="cuda")
        self.m[mod].function("pin_state_values").launch((1,), (1,), [ptr(out)])
        return out.cpu().numpy()

    # ------------------------------------------------------------- integration
    def integrate(self, voxels, coords, depth, rgb, inv12, nmap=None):
        """One update_map_with_colour_kernel (nmap None) or
        update_map_weighted_kernel launch over the blocks `coords`, whose
        voxels (REF_VOXEL records, 512 per block, in that order) are updated."""
        import oracle as O
        import torch
        cu, n = self.cu, len(coords)
        self.set_state("fusion", 1 << 15, max(n, 1) + 1024, max(n, 1))
        vox = torch.from_numpy(np.ascontiguousarray(voxels).view(np.uint8).copy()).cuda()
        ent = np.zeros(n, O.REF_ENTRY)
        ent["ptr"] = 512 * np.arange(n)
        ent["offset"] = -1
        ent["pos"] = coords
        dent = torch.from_numpy(ent.view(np.uint8).copy()).cuda()
        dd = torch.from_numpy(np.ascontiguousarray(depth, np.float32)).cuda()
        dc = torch.from_numpy(np.ascontiguousarray(rgb, np.uint8)).cuda()
        vp = C.c_void_p
        storage = cu.struct_bytes((vp, 0), (vp, 0), (vp, 0), (vp, 0), (vp, vox.data_ptr()), (vp, 0))

        def view(t, step):
            return cu.struct_bytes((vp, t.data_ptr()), (C.c_size_t, step), (C.c_int, P.W), (C.c_int, P.H))

        pose = cu.struct_bytes(*[(C.c_float, float(x)) for x in inv12])
        K = [C.c_float(P.FX), C.c_float(P.FY), C.c_float(P.CX), C.c_float(P.CY)]
        if nmap is None:
            k = self.m["fusion"].function("update_map_with_colour_kernel")
            params = [storage, ptr(dent), C.c_uint(n), view(dd, P.W * 4), view(dc, P.W * 3), pose, *K]
        else:
            dn = torch.from_numpy(np.ascontiguousarray(nmap, np.float32)).cuda()
            k = self.m["fusion"].function("update_map_weighted_kernel")
            params = [storage, ptr(dent), C.c_uint(n), view(dd, P.W * 4), view(dn, P.W * 16), view(dc, P.W * 3), pose,
                      *K]
        if n:
            k.launch((n,), (8, 8), params)
        return vox.cpu().numpy().view(O.REF_VOXEL).reshape(n, 512)

    # ------------------------------------------------------------- raycast
    def raycast(self, dump, visible, T):
        """create_rendering_blocks + raycast at pose T over a map in the
        reference's chained-table layout."""
        import oracle as O
        import torch
        cu = self.cu
        nb, ne, nbk = dump["size"]
        # findEntry walks a bucket's excess chain while offset_ > 0
        # (map_struct.cu:365-380): check on the host that every chain stays in
        # the table and ends, and every block lies inside the voxel array
        tab = dump["table"]
        for i in range(nbk):
            j, steps = i, 0
            while tab[j]["offset"] > 0:
                j = nbk + int(tab[j]["offset"]) - 1
                steps += 1
                assert j < ne and steps <= ne - nbk, "excess chain leaves the table or loops"
        live = tab["ptr"][tab["ptr"] != -1]
        assert np.all((live >= 0) & (live % 512 == 0) & (live + 512 <= nb * 512)), "block outside the voxel array"
        self.set_state("raycast", nbk, ne, nb)
        vox = torch.from_numpy(dump["voxels"].view(np.uint8).copy()).cuda()
        table = torch.from_numpy(dump["table"].view(np.uint8).copy()).cuda()
        # the visible list as HashEntry records (the z-range pass reads pos_ and ptr_ != -1)
        where = {tuple(e["pos"].tolist()): i for i, e in enumerate(dump["table"]) if e["ptr"] != -1}
        vis = dump["table"][[where[tuple(c)] for c in np.asarray(visible).tolist()]].copy()
        dvis = torch.from_numpy(vis.view(np.uint8).copy()).cuda()
        zc, zr = P.W // 8, P.H // 8
        zx = torch.full((zr, zc), 100.0, dtype=torch.float32, device="cuda")  # zrange_x.setTo(100), ray_tracing.cu:239
        zy = torch.zeros((zr, zc), dtype=torch.float32, device="cuda")
        count = torch.zeros(1, dtype=torch.int32, device="cuda")
        # rendering blocks: the fill pass reads up to 3 past the count
        # (split_and_fill_rendering_blocks_kernel's grid rounds the count up to
        # a multiple of 4, ray_tracing.cu:271-274, :194-196); the reference
        # leaves whatever an earlier frame wrote there, here every record
        # starts as an empty box that fills no cell
        blocks = np.zeros(REF_BLOCKS, RENDERING_BLOCK)
        blocks["upper_left"] = 32767
        blocks["lower_right"] = -1
        dblk = torch.from_numpy(blocks.view(np.uint8).copy()).cuda()
        inv = torch.from_numpy(P.f12(P.pose_inv(T))).cuda()
        fwd = torch.from_numpy(P.f12(T)).cuda()
        f = C.c_float
        args = [C.c_int(zc), C.c_int(zr), ptr(inv), f(P.FX), f(P.FY), f(P.CX), f(P.CY), ptr(count), C.c_uint(len(vis)),
                ptr(dvis), ptr(zx), ptr(zy), C.c_int(zc), C.c_int(zr), ptr(dblk)]
        n = len(vis)
        self.m["raycast"].function("pin_rendering_blocks").launch(((n + 1023) // 1024,), (1024,), args)
        nr = int(count.cpu().item())
        if nr:
            self.m["raycast"].function("pin_fill_rendering_blocks").launch((int(np.ceil(nr / 4.0)), 4), (16, 16), args)
        vmap = torch.empty((P.H, P.W, 4), dtype=torch.float32, device="cuda")
        self.m["raycast"].function("pin_raycast").launch(
            ((P.W + 3) // 4, (P.H + 7) // 8), (4, 8),
            [ptr(vox), ptr(table), ptr(vmap), C.c_int(P.W), C.c_int(P.H), ptr(zx), ptr(zy), C.c_int(zc), C.c_int(zr),
             f(np.float32(1.0) / np.float32(P.FX)), f(np.float32(1.0) / np.float32(P.FY)), f(P.CX), f(P.CY), ptr(fwd),
             ptr(inv)])
        z = np.stack([zx.cpu().numpy(), zy.cpu().numpy()], axis=-1)
        return z, vmap.cpu().numpy(), nr

    # ------------------------------------------------------------- rows
    def rows(self, ref, cur, level, T, stddev, cfg):
        import torch
        w, h = P.W >> level, P.H >> level
        fx, fy, cx, cy = (np.float32(v) / np.float32(1 << level) for v in (P.FX, P.FY, P.CX, P.CY))
        img = lambda f, kind: torch.from_numpy(np.ascontiguousarray(f.get(kind, level), np.float32)).cuda()
        rv, rn, ri = img(ref, 0), img(ref, 1), img(ref, 2)
        cv, cn, ci, cdx, cdy = img(cur, 0), img(cur, 1), img(cur, 2), img(cur, 3), img(cur, 4)
        Tt = torch.from_numpy(P.f12(T)).cuda()
        f = C.c_float
        out_icp = torch.full((w * h, 29), float("nan"), dtype=torch.float32, device="cuda")
        out_rgb = torch.full((w * h, 29), float("nan"), dtype=torch.float32, device="cuda")
        grid = ((w * h + 255) // 256,)
        self.m["icp"].function("pin_icp_rows").launch(
            grid, (256,), [ptr(cv), ptr(cn), ptr(rv), ptr(rn), C.c_int(w), C.c_int(h), ptr(Tt), f(fx), f(fy), f(cx),
                           f(cy), f(cfg.icp_angle_thresh), f(cfg.icp_dist_thresh), ptr(out_icp)])
        self.m["rgb"].function("pin_rgb_rows").launch(
            grid, (256,), [ptr(ci), ptr(ri), ptr(rv), ptr(cv), ptr(cdx), ptr(cdy), C.c_int(w), C.c_int(h),
                           f(stddev), ptr(Tt), f(fx), f(fy), f(cx), f(cy), f(np.float32(1) / fx),
                           f(np.float32(1) / fy), ptr(out_rgb)])
        return out_icp.cpu().numpy(), out_rgb.cpu().numpy()


    # ------------------------------------------------------------- image kernels
    def images(self, depth, intensity, level):
        """backProjectDepthK, computeNMapK of its output, computeDerivativeK
        of the intensity; pixels a kernel does not write keep SENTINEL."""
        import torch
        cu, vp = self.cu, C.c_void_p
        h, w = depth.shape
        fx, fy, cx, cy = (np.float32(v) for v in (P.FX, P.FY, P.CX, P.CY))
        for _ in range(level):  # IntrinsicMatrix::pyr_down (intrinsic_matrix.h:33-37)
            fx, fy, cx, cy = (np.float32(0.5) * v for v in (fx, fy, cx, cy))
        K = cu.struct_bytes((C.c_int, w), (C.c_int, h), (C.c_float, fx), (C.c_float, fy), (C.c_float, cx),
                            (C.c_float, cy), (C.c_float, np.float32(1.0) / fx), (C.c_float, np.float32(1.0) / fy))
        dd = torch.from_numpy(np.ascontiguousarray(depth, np.float32)).cuda()
        di = torch.from_numpy(np.ascontiguousarray(intensity, np.float32)).cuda()
        vm = torch.full((h, w, 4), SENTINEL, dtype=torch.float32, device="cuda")
        nm = torch.full((h, w, 4), SENTINEL, dtype=torch.float32, device="cuda")
        dx = torch.full((h, w), SENTINEL, dtype=torch.float32, device="cuda")
        dy = torch.full((h, w), SENTINEL, dtype=torch.float32, device="cuda")
        sz = lambda t, step: cu.struct_bytes((vp, t.data_ptr()), (C.c_size_t, step), (C.c_int, w), (C.c_int, h))
        st = lambda t, step: cu.struct_bytes((vp, t.data_ptr()), (C.c_size_t, step))
        grid, blk = ((w + 7) // 8, (h + 7) // 8), (8, 8)
        mod = self.m["imgproc"]
        mod.function("backProjectDepthK").launch(grid, blk, [sz(dd, w * 4), st(vm, w * 16), K])
        mod.function("computeNMapK").launch(grid, blk, [sz(vm, w * 16), st(nm, w * 16)])
        mod.function("computeDerivativeK").launch(grid, blk, [sz(di, w * 4), st(dx, w * 4), st(dy, w * 4)])
        return {"vmap": P.canonical_nan(vm.cpu().numpy()), "nmap": P.canonical_nan(nm.cpu().numpy()),
                "dx": dx.cpu().numpy(), "dy": dy.cpu().numpy()}

    def shading(self, vmap, nmap, rgb):
        """renderSceneK and renderSceneTexturedK, light at (5, 5, 5) (cuda_imgproc.cu:69-108)."""
        import torch
        cu, vp = self.cu, C.c_void_p
        h, w = vmap.shape[:2]
        dv = torch.from_numpy(np.ascontiguousarray(vmap, np.float32)).cuda()
        dn = torch.from_numpy(np.ascontiguousarray(nmap, np.float32)).cuda()
        dc = torch.from_numpy(np.ascontiguousarray(rgb, np.uint8)).cuda()
        light = cu.struct_bytes((C.c_float, 5.0), (C.c_float, 5.0), (C.c_float, 5.0))
        st = lambda t, step: cu.struct_bytes((vp, t.data_ptr()), (C.c_size_t, step))
        out = []
        for textured in (False, True):
            dst = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
            dsz = cu.struct_bytes((vp, dst.data_ptr()), (C.c_size_t, w * 4), (C.c_int, w), (C.c_int, h))
            grid, blk = ((w + 7) // 8, (h + 7) // 8), (8, 8)
            if textured:
                self.m["imgproc"].function("renderSceneTexturedK").launch(
                    grid, blk, [st(dv, w * 16), st(dn, w * 16), st(dc, w * 3), light, dsz])
            else:
                self.m["imgproc"].function("renderSceneK").launch(grid, blk, [st(dv, w * 16), st(dn, w * 16), light, dsz])
            out.append(dst.cpu().numpy())
        return out

    # ------------------------------------------------------------- marching cubes
    def mesh(self, dump, max_triangles=1 << 20):
        """create_mesh_with_normal and create_mesh_with_colour over a map in
        the reference's chained-table layout: (vertices, normals), (vertices,
        colours), each in canonical order."""
        import torch
        nb, ne, nbk = dump["size"]
        self.set_state("mesh", nbk, ne, nb, max_triangles)
        vox = torch.from_numpy(dump["voxels"].view(np.uint8).copy()).cuda()
        table = torch.from_numpy(dump["table"].view(np.uint8).copy()).cuda()
        out = []
        for select, make, attr in (("pin_mesh_select", "pin_mesh_normals", (np.float32, 3)),
                                   ("pin_mesh_colour_select", "pin_mesh_colour", (np.uint8, 3))):
            blocks = torch.zeros(ne * 20, dtype=torch.uint8, device="cuda")
            nblk = torch.zeros(1, dtype=torch.int32, device="cuda")
            ntri = torch.zeros(1, dtype=torch.int32, device="cuda")
            tri = torch.zeros((max_triangles, 3, 3), dtype=torch.float32, device="cuda")
            att = torch.zeros((max_triangles, 3, 3), dtype=torch.float32 if attr[0] == np.float32 else torch.uint8,
                              device="cuda")
            self.m["mesh"].function(select).launch(((ne + 1023) // 1024,), (1024,),
                                                   [ptr(vox), ptr(table), ptr(blocks), ptr(nblk)])
            bc = int(nblk.cpu().item())
            self.m["mesh"].function(make).launch(((bc + 15) // 16, 16), (8, 8),
                                                 [ptr(vox), ptr(table), ptr(blocks), ptr(nblk), ptr(ntri), ptr(tri),
                                                  ptr(att)])
            n = int(ntri.cpu().item())
            assert n < max_triangles
            v, a = P.sort_triangles(tri[:n].cpu().numpy(), att[:n].cpu().numpy())
            out.append((P.canonical_nan(v), P.canonical_nan(a) if attr[0] == np.float32 else a))
        return out


def ref_state(coords, vox):
    return P.canonical_state(coords, vox["sdf"], vox["weight"], vox["rgb"])


def run_all(ref: Reference, L, O, dep, rgb, poses, oc):
    """Every case on one build of the pin modules; returns the outputs."""
    out = {}
    cfg = P.config(L)
    inv_a, inv_b = P.f12(P.pose_inv(poses[0])), P.f12(P.pose_inv(poses[1]))
    # integration: A into empty blocks, then B (colour and weighted) on top
    va = oc["visible_a"]
    v1 = ref.integrate(np.zeros(len(va) * 512, O.REF_VOXEL).reshape(-1, 512), va, P.depth_m(dep[0]), rgb[0], inv_a)
    s1 = ref_state(va, v1)
    out["s1"] = s1
    prior = {tuple(c): i for i, c in enumerate(s1[0].tolist())}
    vb = oc["visible_b"]
    v1_sorted = v1[np.lexsort((va[:, 2], va[:, 1], va[:, 0]))]
    start = np.zeros((len(vb), 512), O.REF_VOXEL)
    for j, c in enumerate(vb.tolist()):
        if tuple(c) in prior:
            start[j] = v1_sorted[prior[tuple(c)]]
    for mode, nmap in (("colour", None), ("weighted", oc["nmap_b"])):
        v2 = ref.integrate(start.copy(), vb, P.depth_m(dep[1]), rgb[1], inv_b, nmap)
        # blocks the second fuse did not see keep their first-fuse voxels
        coords = np.concatenate([vb, np.array([c for c in s1[0].tolist() if tuple(c) not in
                                               {tuple(x) for x in vb.tolist()}], np.int32).reshape(-1, 3)])
        keep = np.array([prior[tuple(c)] for c in coords[len(vb):].tolist()], np.int64)
        vox = np.concatenate([v2, v1_sorted[keep]]) if len(keep) else v2
        out[f"s2_{mode}"] = ref_state(coords, vox)
    # z-range + raycast over the map after A and B (colour updates)
    om, _ = P.oracle_raycasts(L, O, dep, rgb, poses, ())
    coords, sdf, w, c = om.export()
    nblk = len(coords)
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "map.data"
        L.write_dump(str(path), coords, sdf, w, c, size=(nblk, 2 * nblk + 64, nblk + 32))
        dump = O.parse_ref_dump(path)
    # the voxels at the dump's block positions, with the oracle's exact codes
    st = P.map_state_from_oracle(coords, sdf, w, c)
    by = {tuple(x): i for i, x in enumerate(st[0].tolist())}
    for e in dump["table"]:
        if e["ptr"] == -1:
            continue
        i = by[tuple(e["pos"].tolist())]
        blk = dump["voxels"][e["ptr"]:e["ptr"] + 512]
        blk["sdf"], blk["weight"], blk["rgb"] = st[1][i], st[2][i], st[3][i]
    for k, T in enumerate(P.raycast_poses(poses)):
        z, v, nr = ref.raycast(dump, oc["visible_b"], T)
        out[f"zrange_{k}"], out[f"vmap_{k}"], out[f"render_blocks_{k}"] = z, P.canonical_nan(v), nr
    (out["mesh_normal_v"], out["mesh_normal_n"]), (out["mesh_colour_v"], out["mesh_colour_c"]) = ref.mesh(dump)
    # image kernels and shading on frame B's images
    im = P.oracle_images(L, O, dep, rgb)
    for level in P.LEVELS:
        for k, v in ref.images(im[level]["depth"], im[level]["intensity"], level).items():
            out[f"img_{k}_{level}"] = v
    out["shade"], out["shade_textured"] = ref.shading(im[0]["vmap"], im[0]["nmap"], rgb[1])
    # rows
    fr = P.oracle_frames(L, O, dep, rgb)
    T = P.relative(poses[0], poses[1])
    for level in P.LEVELS:
        for sd in P.STDDEVS:
            icp, pho = ref.rows(fr[0], fr[1], level, T, sd, cfg)
            out[f"icp_{level}"] = icp
            out[f"rgb_{level}_{sd:g}"] = pho
    return out


def compare_with_oracle(L, O, dep, rgb, poses, got) -> dict:
    """Bit-exactness of the oracle on this machine, per case (for the log)."""
    oc = P.oracle_states(L, O, dep, rgb, poses)
    rep = {}
    for k in ("s1", "s2_colour", "s2_weighted"):
        a, b = oc[k], got[k]
        same_blocks = np.array_equal(a[0], b[0])
        rep[k] = {"blocks": int(len(b[0])), "same_blocks": bool(same_blocks)}
        if same_blocks:
            rep[k]["sdf_codes_differing"] = int(np.sum(a[1] != b[1]))
            rep[k]["max_code_diff"] = int(np.abs(a[1].astype(int) - b[1].astype(int)).max())
            rep[k]["weights_differing"] = int(np.sum(a[2].view(np.int32) != b[2].view(np.int32)))
            rep[k]["rgb_differing"] = int(np.sum(a[3] != b[3]))
    _, rays = P.oracle_raycasts(L, O, dep, rgb, poses, P.raycast_poses(poses))
    for k, (z, v) in enumerate(rays):
        rep[f"zrange_{k}"] = bool(np.array_equal(z, got[f"zrange_{k}"]))
        rep[f"vmap_{k}"] = bool(np.array_equal(v.view(np.int32), got[f"vmap_{k}"].view(np.int32)))
    fr = P.oracle_frames(L, O, dep, rgb)
    T = P.relative(poses[0], poses[1])
    for level in P.LEVELS:
        for sd in P.STDDEVS:
            icp, pho = P.oracle_rows(O, fr[0], fr[1], level, T, sd)
            rep[f"icp_{level}"] = bool(np.array_equal(icp.view(np.int32), got[f"icp_{level}"].view(np.int32)))
            rep[f"rgb_{level}_{sd:g}"] = bool(np.array_equal(pho.view(np.int32), got[f"rgb_{level}_{sd:g}"].view(np.int32)))
    om, _ = P.oracle_raycasts(L, O, dep, rgb, poses, ())
    (vn, nn), (vc, cc) = P.oracle_meshes(om)
    rep["mesh"] = {"triangles": int(len(got["mesh_normal_v"])), "oracle_triangles": int(len(vn)),
                   "normal_mesh": bool(len(vn) == len(got["mesh_normal_v"]) and np.array_equal(
                       vn.view(np.int32), got["mesh_normal_v"].view(np.int32)) and np.array_equal(
                       nn.view(np.int32), got["mesh_normal_n"].view(np.int32))),
                   "colour_mesh": bool(len(vc) == len(got["mesh_colour_v"]) and np.array_equal(
                       vc.view(np.int32), got["mesh_colour_v"].view(np.int32)) and np.array_equal(
                       cc, got["mesh_colour_c"]))}
    im = P.oracle_images(L, O, dep, rgb)
    for level in P.LEVELS:
        for k in ("vmap", "nmap", "dx", "dy"):
            a, b = P.interior(im[level][k]), P.interior(got[f"img_{k}_{level}"])
            if k == "vmap":
                a, b = im[level][k], got[f"img_{k}_{level}"]
            rep[f"img_{k}_{level}"] = bool(np.array_equal(a.view(np.int32), b.view(np.int32)))
    s0, s1 = P.oracle_shading(O, dep, rgb, im)
    for name, a, b in (("shade", s0, got["shade"]), ("shade_textured", s1, got["shade_textured"])):
        d = np.abs(a.astype(int) - b.astype(int))
        rep[name] = {"pixels_differing": int(np.sum(d.max(axis=-1) > 0)), "max_diff": int(d.max())}
    return rep


def contraction_report(a: dict, b: dict) -> dict:
    """How far the reference built with nvcc's default contraction is from
    the same source built with every operation rounded as written."""
    rep = {}
    for k in ("s1", "s2_colour", "s2_weighted"):
        rep[k] = {"sdf_codes_differing": int(np.sum(a[k][1] != b[k][1])), "voxels": int(a[k][1].size),
                  "max_code_diff": int(np.abs(a[k][1].astype(int) - b[k][1].astype(int)).max())}
    for k in (0, 1):
        va, vb = a[f"vmap_{k}"], b[f"vmap_{k}"]
        ha, hb = ~np.isnan(va[..., 2]), ~np.isnan(vb[..., 2])
        both = ha & hb
        rep[f"vmap_{k}"] = {"hit_masks_differing": int(np.sum(ha != hb)), "hits": int(ha.sum()),
                            "max_abs_z_diff_m": float(np.abs(va[..., 2][both] - vb[..., 2][both]).max())
                            if both.any() else 0.0,
                            "vertices_differing": int(np.sum(np.any(va[both] != vb[both], axis=-1)))}
    rep["mesh_triangles"] = [int(len(a["mesh_normal_v"])), int(len(b["mesh_normal_v"]))]
    for k in ("img_vmap_0", "img_nmap_0", "img_dx_0", "img_dy_0", "shade", "shade_textured"):
        rep[k] = {"values_differing": int(np.sum(a[k].view(np.uint8 if a[k].dtype == np.uint8 else np.int32) !=
                                                 b[k].view(np.uint8 if b[k].dtype == np.uint8 else np.int32)))}
    for k in a:
        if k.startswith(("icp_", "rgb_")):
            x, y = a[k], b[k]
            rep[k] = {"pixels_differing": int(np.sum(np.any(x.view(np.int32) != y.view(np.int32), axis=1))),
                      "pixels": int(len(x)), "flags_differing": int(np.sum(x[:, 28] != y[:, 28]))}
    return rep


def main() -> None:
    import torch
    out_path = Path(sys.argv[1]) if len(sys.argv) > 1 else ROOT / "tests" / "golden" / "ref_kernels.npz"
    assert torch.cuda.is_available(), "needs a CUDA GPU"
    torch.zeros(1, device="cuda")  # the primary context, current on this thread
    from libfusion_gb300 import build as B
    B.build()
    import libfusion_gb300 as L
    import oracle as O
    O.build()
    K = P.intrinsics(L)
    sc = L.SynthScene(seed=0)
    dep, rgb, poses = [], [], []
    for k in P.FRAMES:
        d, c = sc.render(K, k)
        torch.cuda.synchronize()
        dep.append(d.cpu().numpy())
        rgb.append(c.cpu().numpy())
        poses.append(sc.pose(k))
    sc.close()
    dep, rgb, poses = np.stack(dep), np.stack(rgb), np.stack(poses)
    # the oracle's sinf arguments (the normal-weighted update), recorded, with
    # CUDA's sinf of each: the pin test installs them as the oracle's table
    O.trans_record(True)
    oc = P.oracle_states(L, O, dep, rgb, poses)
    O.trans_record(False)
    sin_x = O.trans_recorded(O.TRANS_SIN)
    sin_y = torch.sin(torch.from_numpy(sin_x).cuda()).cpu().numpy()

    exact = Reference("")
    exact.set_state("fusion", 1 << 15, 1 << 14, 1 << 13)
    vals = exact.state_values("fusion")
    assert vals[0] == P.TAU, (vals, P.TAU)
    got = run_all(exact, L, O, dep, rgb, poses, oc)
    fmad = run_all(Reference("_fmad"), L, O, dep, rgb, poses, oc)
    report = {"oracle_here": compare_with_oracle(L, O, dep, rgb, poses, got),
              "default_contraction_vs_as_written": contraction_report(got, fmad),
              "state_values": [float(x) for x in vals]}
    print(json.dumps(report, indent=1))

    fx = {"depth_u16": dep, "rgb": rgb, "poses": poses, "frame_digest": np.array(P.frame_digest(
        P.oracle_frames(L, O, dep, rgb))), "sin_x": sin_x, "sin_y": sin_y}
    for k in ("s1", "s2_colour", "s2_weighted"):
        coords, code, w, c = got[k]
        chosen = P.choose_subset(coords)
        idx = P.subset_rows(coords, chosen)
        fx[f"{k}_coords"] = coords
        fx[f"{k}_digest"] = np.array(P.digest(coords, code, w, c))
        fx[f"{k}_subset"] = chosen
        fx[f"{k}_subset_code"], fx[f"{k}_subset_weight"], fx[f"{k}_subset_rgb"] = code[idx], w[idx], c[idx]
    for k in (0, 1):
        fx[f"zrange_{k}"], fx[f"vmap_{k}"] = got[f"zrange_{k}"], got[f"vmap_{k}"]
        fx[f"render_blocks_{k}"] = np.array(got[f"render_blocks_{k}"])
    for level in P.LEVELS:
        n = (P.W >> level) * (P.H >> level)
        s = P.sample_pixels(n, level)
        for k in [f"icp_{level}"] + [f"rgb_{level}_{sd:g}" for sd in P.STDDEVS]:
            fx[f"{k}_digest"] = np.array(P.digest(got[k]))
            fx[f"{k}_sample"] = got[k][s]
            fx[f"{k}_found"] = np.packbits(got[k][:, 28] != 0)
    for k in ("normal", "colour"):
        v, att = got[f"mesh_{k}_v"], got[f"mesh_{k}_{k[0]}"]
        s = P.sample_triangles(len(v))
        fx[f"mesh_{k}_digest"] = np.array(P.digest(v, att))
        fx[f"mesh_{k}_count"] = np.array(len(v))
        fx[f"mesh_{k}_sample_v"], fx[f"mesh_{k}_sample_a"] = v[s], att[s]
    for level in P.LEVELS:
        fx[f"img_vmap_{level}_digest"] = np.array(P.digest(got[f"img_vmap_{level}"]))
        fx[f"img_nmap_{level}_digest"] = np.array(P.digest(P.interior(got[f"img_nmap_{level}"])))
        fx[f"img_nmap_{level}_border_unwritten"] = np.array(bool(
            np.all(got[f"img_nmap_{level}"][-1] == SENTINEL) and np.all(got[f"img_nmap_{level}"][:, -1] == SENTINEL)))
        fx[f"img_dx_{level}"], fx[f"img_dy_{level}"] = got[f"img_dx_{level}"], got[f"img_dy_{level}"]
    fx["shade"], fx["shade_textured"] = got["shade"], got["shade_textured"]
    fx["report"] = np.array(json.dumps(report))
    out_path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(out_path, **fx)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
