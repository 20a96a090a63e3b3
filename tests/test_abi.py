"""The C-ABI boundary: the sm_103a library builds, loads and exports every entry point the
public header declares; argument errors come back as status codes (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER_DIR = os.path.join(ROOT, "include")


def declared_functions():
    names = []
    for h in sorted(os.listdir(HEADER_DIR)):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(HEADER_DIR, h)).read()
        names += re.findall(r"^RT_API\s+[\w\s\*]+?\b(\w+)\s*\(", text, flags=re.M)
    return names


@pytest.fixture(scope="module")
def built_lib():
    from rendu_gb300 import build

    return build.build()


def test_header_declares_the_reference_api():
    names = set(declared_functions())
    # Raycaster (Raycaster.hpp:51-97) and PathTracer (PathTracer.hpp:18-29) counterparts.
    for n in ["rt_create", "rt_add_mesh", "rt_update_hierarchy", "rt_intersect", "rt_intersect_any", "rt_visible",
              "rt_prim_info", "rt_destroy", "pt_scene_create", "pt_scene_commit", "pt_render"]:
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", built_lib], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    lib = C.CDLL(built_lib)
    for n in declared_functions():
        getattr(lib, n)


def test_argument_errors_are_status_codes(built_lib):
    import rendu_gb300._lib as L

    lib = L.lib()
    assert lib.rt_create(None, 0) == L.RT_ERR_ARG
    assert lib.rt_add_mesh(None, None, 0, None, 0, None, None) == L.RT_ERR_ARG
    assert lib.rt_intersect(None, None, 0, None, None, 0) == L.RT_ERR_ARG
    assert lib.rt_update_hierarchy(None) == L.RT_ERR_ARG
    assert lib.pt_render(None, None, 1, 1, 0, None, 1, 1, 3, None, 0) == L.RT_ERR_ARG
    assert lib.rt_last_error() != b""


def test_no_device_is_an_error_not_a_crash(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import rendu_gb300._lib as L

    h = C.c_void_p()
    assert L.lib().rt_create(C.byref(h), 0) == L.RT_ERR_CUDA
    assert b"not available" in L.lib().rt_last_error()
