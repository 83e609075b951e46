"""Minimal CUDA driver API access (ctypes over libcuda) for the reference-kernel
pin modules in oracle/_ref/*.cubin: load a module, find its kernels, launch
them.  Test infrastructure only, used by tests/golden/make_kernel_golden.py.
Device memory comes from torch tensors; the launches run on the legacy
default stream and every launch is followed by a synchronisation, so a fault
is reported at the launch that caused it."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_cu = None


def _lib():
    global _cu
    if _cu is None:
        _cu = C.CDLL("libcuda.so.1")
        _cu.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        _cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        _cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        _cu.cuModuleGetFunctionCount.argtypes = [C.POINTER(C.c_uint), C.c_void_p]
        _cu.cuModuleEnumerateFunctions.argtypes = [C.POINTER(C.c_void_p), C.c_uint, C.c_void_p]
        _cu.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), C.c_void_p]
        _cu.cuFuncGetParamInfo.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        _cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                       C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        _cu.cuModuleUnload.argtypes = [C.c_void_p]
        _check(_cu.cuInit(0), "cuInit")
    return _cu


def _check(rc: int, what: str) -> None:
    if rc != 0:
        s = C.c_char_p()
        _cu.cuGetErrorString(rc, C.byref(s))
        raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'?').decode()})")


class Module:
    """A loaded device module.  torch must have initialised CUDA first, so
    that its primary context is current on this thread."""

    def __init__(self, path: Path):
        self.path = Path(path)
        if not self.path.exists():
            raise FileNotFoundError(f"{self.path}: build it with oracle/ref_pin/build_kernels.sh")
        cu = _lib()
        self.h = C.c_void_p()
        _check(cu.cuModuleLoad(C.byref(self.h), str(self.path).encode()), f"cuModuleLoad {self.path.name}")

    def names(self) -> dict[str, C.c_void_p]:
        """Every kernel of the module by its (mangled) name."""
        cu = _lib()
        n = C.c_uint()
        _check(cu.cuModuleGetFunctionCount(C.byref(n), self.h), "cuModuleGetFunctionCount")
        fs = (C.c_void_p * n.value)()
        _check(cu.cuModuleEnumerateFunctions(fs, n.value, self.h), "cuModuleEnumerateFunctions")
        out = {}
        for f in fs:
            s = C.c_char_p()
            _check(cu.cuFuncGetName(C.byref(s), C.c_void_p(f)), "cuFuncGetName")
            out[s.value.decode()] = C.c_void_p(f)
        return out

    def function(self, name: str) -> "Kernel":
        """An extern "C" kernel by name, or the one kernel whose mangled name
        contains `name` as an identifier."""
        cu = _lib()
        f = C.c_void_p()
        if cu.cuModuleGetFunction(C.byref(f), self.h, name.encode()) == 0:
            return Kernel(f, name)
        tag = f"{len(name)}{name}"  # Itanium mangling: <length><identifier>
        hits = [(k, v) for k, v in self.names().items() if tag in k]
        if len(hits) != 1:
            raise KeyError(f"{name}: {len(hits)} kernels match in {self.path.name}")
        return Kernel(hits[0][1], hits[0][0])

    def close(self) -> None:
        if self.h:
            _lib().cuModuleUnload(self.h)
            self.h = C.c_void_p()


class Kernel:
    def __init__(self, f: C.c_void_p, name: str):
        self.f, self.name = f, name

    def param_sizes(self) -> list[int]:
        cu = _lib()
        sizes = []
        while True:
            off, size = C.c_size_t(), C.c_size_t()
            if cu.cuFuncGetParamInfo(self.f, len(sizes), C.byref(off), C.byref(size)) != 0:
                return sizes
            sizes.append(size.value)

    def launch(self, grid, block, params: list) -> None:
        """params: one ctypes object per kernel parameter (a c_int, c_float,
        c_void_p, or a bytes buffer of the parameter's size for a struct)."""
        cu = _lib()
        sizes = self.param_sizes()
        if len(sizes) != len(params):
            raise ValueError(f"{self.name}: {len(sizes)} parameters, {len(params)} given")
        for i, (p, s) in enumerate(zip(params, sizes)):
            if C.sizeof(p) != s:
                raise ValueError(f"{self.name}: parameter {i} is {s} bytes, {C.sizeof(p)} given")
        arr = (C.c_void_p * len(params))(*[C.cast(C.pointer(p), C.c_void_p) for p in params])
        g = tuple(grid) + (1,) * (3 - len(grid))
        b = tuple(block) + (1,) * (3 - len(block))
        _check(cu.cuLaunchKernel(self.f, *g, *b, 0, None, arr, None), f"launch {self.name}")
        _check(cu.cuCtxSynchronize(), f"after {self.name}")


def struct_bytes(*fields) -> C.Array:
    """A packed parameter struct from (ctype, value) fields, each placed at its
    natural alignment (the layout a kernel parameter of that struct has)."""
    buf, off = bytearray(), 0
    for ct, v in fields:
        a = C.alignment(ct)
        pad = (-off) % a
        buf += b"\0" * pad
        off += pad
        x = ct(v) if not isinstance(v, ct) else v
        buf += bytes(x)
        off += C.sizeof(ct)
    align = max(C.alignment(ct) for ct, _ in fields)
    buf += b"\0" * ((-off) % align)
    return (C.c_char * len(buf)).from_buffer_copy(bytes(buf))
