"""The C ABI library loads without a GPU, exports every function include/*.h
declares, and the ctypes structures match the header's layout."""
import ctypes as ct
import pathlib
import re
import subprocess

ROOT = pathlib.Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(elbm_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_entry_points():
    names = declared_functions()
    assert {"elbm_create", "elbm_destroy", "elbm_level_register", "elbm_set_links", "elbm_level_step",
            "elbm_upload_level", "elbm_download_level", "elbm_last_error_string"} <= names


def test_library_exports_every_declared_symbol(pkg, built_lib):
    lib = ct.CDLL(str(built_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes binding covers every declared function
    assert declared_functions() <= set(pkg.capi.SIGNATURES)


def test_struct_layout_matches_header(pkg, tmp_path):
    cap = pkg.capi
    src = tmp_path / "layout.c"
    src.write_text(f"""
#include <stddef.h>
#include <stdio.h>
#include "{ROOT / 'include' / 'elbm_gb300.h'}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu\\n", sizeof(elbm_d3q27_params), offsetof(elbm_d3q27_params, outlet_type),
         offsetof(elbm_d3q27_params, fs_feq), offsetof(elbm_d3q27_params, outl_feq), sizeof(elbm_stats));
  printf("%zu %zu %zu\\n", offsetof(elbm_stats, status), offsetof(elbm_stats, kernel_ms), sizeof(elbm_d3q39_params));
  return 0;
}}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    P, S = cap.D3Q27Params, cap.Stats
    expect = [ct.sizeof(P), P.outlet_type.offset, P.fs_feq.offset, P.outl_feq.offset, ct.sizeof(S), S.status.offset,
              S.kernel_ms.offset, ct.sizeof(cap.D3Q39Params)]
    assert list(map(int, out)) == expect


def test_more_struct_layouts(pkg, tmp_path):
    """The D3Q39 boundary block and the Plot3D header keep the header's layout in ctypes."""
    cap = pkg.capi
    src = tmp_path / "layout39.c"
    src.write_text(f"""
#include <stddef.h>
#include <stdio.h>
#include "{ROOT / 'include' / 'elbm_gb300.h'}"
int main(void) {{
  printf("%zu %zu %zu %zu %zu\\n", sizeof(elbm_d3q39_bc), offsetof(elbm_d3q39_bc, fs_u), offsetof(elbm_d3q39_bc, fs_temp),
         offsetof(elbm_d3q39_params, su_lm), sizeof(elbm_plot3d_header));
  return 0;
}}
""")
    exe = tmp_path / "layout39"
    subprocess.run(["gcc", str(src), "-o", str(exe)], check=True)
    out = list(map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()))
    B, P = cap.D3Q39Bc, cap.D3Q39Params
    assert out == [ct.sizeof(B), B.fs_u.offset, B.fs_temp.offset, P.su_lm.offset, ct.sizeof(cap.Plot3DHeader)]


def test_errors_without_a_context_or_a_gpu(pkg, built_lib):
    """Entry points return ELBM_E_* codes and never abort: a null context, host-only set-up
    helpers with bad sizes, and (where this machine has no GPU) context creation."""
    cap = pkg.capi
    lib = ct.CDLL(str(built_lib))
    vp = ct.c_void_p
    lib.elbm_level_step.argtypes = [vp, ct.c_int, ct.c_int, vp]
    assert lib.elbm_level_step(None, 0, 1, None) == cap.ELBM_E_ARG
    lib.elbm_last_error_string.restype = ct.c_char_p
    lib.elbm_last_error_string.argtypes = [vp]
    assert lib.elbm_last_error_string(None) == b"null context"
    lib.elbm_mark_triangles.argtypes = [ct.c_int, ct.c_int, ct.c_int, vp, ct.c_double, ct.c_int, vp, vp]
    assert lib.elbm_mark_triangles(0, 4, 4, None, 1.0, 1, None, None) == cap.ELBM_E_ARG
    import numpy as np
    st = np.zeros((39, 3, 3, 3), np.int32)
    with __import__("pytest").raises(cap.ElbmError):
        cap.links39_tables(st, 8, 0, 1, [1] * 8, [1] * 8)  # periodic mask out of range
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        out = vp()
        lib.elbm_create.argtypes = [ct.c_int, ct.POINTER(vp)]
        assert lib.elbm_create(0, ct.byref(out)) == cap.ELBM_E_CUDA and not out.value
