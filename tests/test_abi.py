"""The C ABI library loads and exports every symbol include/nairn_mpm_gpu.h declares."""
import ctypes
import os
import re

from conftest import ROOT


def header_symbols():
    src = open(os.path.join(ROOT, "include", "nairn_mpm_gpu.h")).read()
    return sorted(set(re.findall(r"\b(mpmgpu_[a-z_]+)\s*\(", src)))


def test_header_lists_expected_entry_points():
    syms = header_symbols()
    for s in ("mpmgpu_create", "mpmgpu_step", "mpmgpu_upload_particles", "mpmgpu_download_particles",
              "mpmgpu_destroy", "mpmgpu_last_error"):
        assert s in syms


def test_library_exports_header_symbols(gpu_lib):
    lib = ctypes.CDLL(os.path.join(ROOT, "nairn-mpm-fea_gb300", "lib", "libnairn_mpm_gb300.so"))
    for s in header_symbols():
        assert hasattr(lib, s), s
    assert lib.mpmgpu_abi_version() == 1


def test_create_rejects_bad_options_without_gpu_work(gpu_lib):
    """Argument validation happens on the host before any device call."""
    import ctypes as C
    from nairn_gb300 import abi, model
    m = model.cantilever_2d(nx=6, ny=3, steps=5)
    b = abi.Bound()
    g = abi.grid_struct(m, b)
    o = abi.options_struct(m)
    o.shape = 4  # finite GIMP is not implemented
    h = C.c_void_p()
    st = gpu_lib.mpmgpu_create(C.byref(g), C.byref(o), C.byref(h))
    assert st == 2 and not h.value
    assert b"shape" in gpu_lib.mpmgpu_last_error(None)
    m3 = model.taylor_3d(radius=1.0, length=2.0, cell=0.5, steps=5)
    g3 = abi.grid_struct(m3, b)
    o3 = abi.options_struct(m3)
    o3.shape = model.SHAPE_QCPDI  # qCPDI is 2D only, as in the reference
    st = gpu_lib.mpmgpu_create(C.byref(g3), C.byref(o3), C.byref(h))
    assert st == 2 and not h.value
    assert b"qCPDI" in gpu_lib.mpmgpu_last_error(None)
    o = abi.options_struct(m, p2g=3)  # node sums: atomic (0), deterministic (1) or untiled (2) only
    st = gpu_lib.mpmgpu_create(C.byref(g), C.byref(o), C.byref(h))
    assert st == 2 and not h.value
    assert b"p2g" in gpu_lib.mpmgpu_last_error(None)


def test_ctypes_structs_match_the_header(tmp_path):
    """Every POD struct of the header has the size and field offsets of its
    ctypes mirror (compiled with the host C compiler from the header)."""
    import shutil
    import subprocess
    import sys
    if shutil.which("gcc") is None:
        import pytest
        pytest.skip("no host C compiler")
    sys.path.insert(0, os.path.join(ROOT, "nairn-mpm-fea_gb300", "python"))
    from nairn_gb300 import abi
    structs = [v for k, v in vars(abi).items()
               if k.startswith("MpmGpu") and isinstance(v, type) and issubclass(v, ctypes.Structure)]
    assert len(structs) >= 11
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "nairn_mpm_gpu.h"', "int main(void) {"]
    expect = []
    for s in structs:
        lines.append(f'printf("%zu\\n", sizeof({s.__name__}));')
        expect.append(ctypes.sizeof(s))
        for name, *_ in s._fields_:
            cname = name[:-1] if name.endswith("_") else name  # Python keywords carry a trailing _
            lines.append(f'printf("%zu\\n", offsetof({s.__name__}, {cname}));')
            expect.append(getattr(s, name).offset)
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect


def test_host_state_step_validates_without_gpu_work(gpu_lib):
    """mpmgpu_step_host refuses a missing context or particle set on the host."""
    import ctypes as C
    from nairn_gb300 import abi
    ps = abi.MpmGpuParticles()
    assert gpu_lib.mpmgpu_step_host(None, C.byref(ps), 1, C.c_double(0.0)) == 1
    assert gpu_lib.mpmgpu_step_host(None, None, 1, C.c_double(0.0)) == 1
