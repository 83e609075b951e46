"""The header-only C++ shim (include/gbfusion.hpp) compiles against the C ABI
and its host-only calls work without a GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

SRC = r'''
#include "gbfusion.hpp"
#include <cstdio>
int main() {
    fusion::IntrinsicMatrix K(640, 480, 525.f, 525.f, 319.5f, 239.5f);
    fusion::IntrinsicMatrix K2 = K.pyr_down();
    gbf_config c = fusion::default_config();
    gbf_intrinsics k = K.c();
    uint64_t bytes = 0;
    fusion::check(gbf_session_bytes(&c, &k, &bytes), "bytes");
    bool threw = false;
    try { c.num_levels = 9; fusion::check(gbf_session_bytes(&c, &k, &bytes), "bad"); }
    catch (const fusion::Error &e) { threw = e.status == GBF_ERR_INVALID_ARG; }
    printf("%d %d %.4f %llu %d\n", K2.width, K2.height, K2.cx, (unsigned long long)bytes, threw ? 1 : 0);
    return 0;
}
'''


def test_cpp_shim_compiles_and_runs(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    from libfusion_gb300 import build as B
    lib = B.build()
    src = tmp_path / "t.cpp"
    src.write_text(SRC)
    exe = tmp_path / "t"
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run([gxx, "-std=c++17", "-I", str(ROOT / "include"), "-I", cuda_inc, str(src), "-o", str(exe),
                        str(lib), f"-Wl,-rpath,{lib.parent}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out[0] == "320" and out[1] == "240" and out[2] == "159.7500"
    assert int(out[3]) > 200000 * 512 * 10 and out[4] == "1"
