"""The C-ABI library: loads, exports every symbol include/faces_gb300.h
declares, and reports argument errors without touching a GPU."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in sorted(os.listdir(os.path.join(ROOT, "include")))
           if h.endswith(".h")]


def declared():
    names = []
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\**\s*(faces_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared()
    for must in ("faces_create", "faces_destroy", "faces_share", "faces_layout", "faces_check"):
        assert must in names


def test_library_exports_every_declared_symbol(faces_lib):
    L = ctypes.CDLL(faces_lib.library_path)
    missing = [n for n in declared() if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", faces_lib.library_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (faces_\w+)", out))
    assert set(declared()) <= exported


def test_argument_errors_without_gpu(faces_lib):
    F = faces_lib
    L = F.lib()
    h = ctypes.c_void_p()
    for args in [(1, 1, 1, 4, 4, 4, 1, 0), (0, 1, 1, 4, 4, 4, 5, 0), (1, 1, 1, 4, 0, 4, 5, 0),
                 (1, 1, 1, 4, 4, 4, 5, 0x200), (1, 1, 1, 4, 4, 4, 5, 0x80 | 0x2)]:
        assert L.faces_create(ctypes.byref(h), *args) == -1
        assert L.faces_last_error()
    assert L.faces_share(None, None, 1, None) == -1
    assert L.faces_run_host_many(None, 1, None, None, 1, 1, None) == -1
    assert L.faces_destroy(None) == 0
    with pytest.raises(F.FacesError):
        F.Faces(1, 1, 1, 2, 2, 2, 1)


def test_executable_prints_reference_header_lines(faces_lib):
    exe = faces_lib.exe_path
    if not os.path.isfile(exe):
        pytest.skip("executable not built")
    r = subprocess.run([exe], input="1 1 1 4 4 4 5 1 2 -5\n", capture_output=True, text=True, timeout=120)
    lines = r.stdout.splitlines()
    assert lines[:3] == ["1 1 1 tasks", "4 4 4 local elements of size 5",
                         "1 face inits x 2 element inits x 5 shares without compute kernels"]
    r = subprocess.run([exe], input="1 2\n", capture_output=True, text=True, timeout=60)
    assert r.returncode == 2


def test_struct_layouts_match_header(faces_lib, tmp_path):
    """The ctypes mirrors of faces_job and faces_serve_stats have the C layout."""
    F = faces_lib
    src = tmp_path / "layout.c"
    src.write_text(
        "#include <stdio.h>\n#include <stddef.h>\n#include \"faces_gb300.h\"\n"
        "int main(void) {\n"
        "  printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(faces_job), offsetof(faces_job, seed),\n"
        "         offsetof(faces_job, host_in), sizeof(faces_serve_stats),\n"
        "         offsetof(faces_serve_stats, point_shares), offsetof(faces_serve_stats, queued));\n"
        "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == [ctypes.sizeof(F.FacesJob), F.FacesJob.seed.offset, F.FacesJob.host_in.offset,
                   ctypes.sizeof(F.ServeStats), F.ServeStats.point_shares.offset, F.ServeStats.queued.offset]


def test_batch_and_server_errors_without_gpu(faces_lib):
    """Without a GPU, creating a batch or a server fails with FACES_ECUDA and a
    message; NULL handles are rejected or accepted as documented."""
    F = faces_lib
    L = F.lib()
    h = ctypes.c_void_p()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    assert L.faces_batch_create(ctypes.byref(h)) == -2 and L.faces_last_error()
    assert L.faces_server_create(ctypes.byref(h), 1 << 30, 0, 0) == -2 and L.faces_last_error()
    assert L.faces_server_create(ctypes.byref(h), 0, 0, 0) == -1
    assert L.faces_batch_commit(None) == -1
    assert L.faces_batch_destroy(None) == 0
    assert L.faces_server_destroy(None) == 0
    assert L.faces_server_poll(None, 0) == -1
    with pytest.raises(F.FacesError):
        F.Server(1 << 30)
