"""CPU checks of the C ABI: the library loads, exports every function include/swgpu.h declares, and the
Python mirrors of the structs have the C layouts. No GPU calls."""
import ctypes
import os
import re

from sqwheel import abi, gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(sw\w*)\s*\(", text, re.M)))


def test_header_symbols_exported(built_libs):
    names = sorted(declared_functions("swgpu.h") + declared_functions("swlearn.h"))
    assert len(names) >= 30
    lib = ctypes.CDLL(gpu.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    # The Python binding binds exactly the declared set.
    assert sorted(gpu.EXPORTED) == names


def test_struct_layouts_match(built_libs):
    sizes = gpu.abi_layout()
    assert sizes == [s for _, s in abi.LAYOUT_ORDER], list(zip([n for n, _ in abi.LAYOUT_ORDER], sizes))
    assert abi.SURFACE_DESC.itemsize == 136
    assert abi.DRAW_CMD.itemsize == 72
    assert abi.DIR_LIGHTMAP_ELEMENT.itemsize == 40


def test_create_without_gpu_fails_cleanly(built_libs):
    """On a machine without a device sw_create must return an error, never abort."""
    try:
        import torch
        if torch.cuda.is_available():
            return
    except Exception:
        pass
    lib = gpu.load_library()
    ci = abi.CreateInfo()
    ci.abi_version = abi.SWGPU_ABI_VERSION
    ctx = ctypes.c_void_p()
    r = lib.sw_create(ctypes.byref(ci), ctypes.byref(ctx))
    assert r == abi.SW_ERR_NO_DEVICE
    assert not ctx.value


def test_bad_abi_version_rejected(built_libs):
    lib = gpu.load_library()
    ci = abi.CreateInfo()
    ci.abi_version = 999
    ctx = ctypes.c_void_p()
    assert lib.sw_create(ctypes.byref(ci), ctypes.byref(ctx)) == abi.SW_ERR_INVALID_ARGUMENT
    assert lib.sw_create(None, ctypes.byref(ctx)) == abi.SW_ERR_INVALID_ARGUMENT
    assert lib.sw_destroy(None) == abi.SW_ERR_INVALID_ARGUMENT
