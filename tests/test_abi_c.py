"""The C-ABI used from plain C and C++ without Python: a program that includes only
include/rendu_gb300.h compiles as C11 and as C++17, links against the library, and gets
status codes and messages back for invalid arguments and for a missing device (no GPU
needed). This is the boundary a Rendu maintainer binds from the reference's C++ classes."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

PROGRAM = r"""
#include "rendu_gb300.h"
#include <stdio.h>
#include <string.h>

int main(void) {
    /* invalid arguments are status codes, with a message */
    if (rt_create(NULL, 0) != RT_ERR_ARG) return 1;
    if (strlen(rt_last_error()) == 0) return 2;
    if (rt_add_mesh(NULL, NULL, 0, NULL, 0, NULL, NULL) != RT_ERR_ARG) return 3;
    if (rt_update_hierarchy(NULL) != RT_ERR_ARG) return 4;
    if (rt_intersect(NULL, NULL, 0, NULL, NULL, 0) != RT_ERR_ARG) return 5;
    if (rt_intersect_any(NULL, NULL, 0, NULL, NULL, 0) != RT_ERR_ARG) return 6;
    if (rt_destroy(NULL) != RT_OK && rt_destroy(NULL) != RT_ERR_ARG) return 7;
    /* the record layouts the reference-side binding relies on */
    if (sizeof(rt_ray) != 32 || sizeof(rt_hit) != 16) return 8;
    /* without a usable device, creation fails with a status, not a crash */
    rt_ctx *ctx = NULL;
    int r = rt_create(&ctx, 0);
    if (r == RT_OK) {
        rt_destroy(ctx);
        printf("device\n");
        return 0;
    }
    printf("no-device %d %s\n", r, rt_last_error());
    return r == RT_ERR_CUDA ? 0 : 9;
}
"""


@pytest.fixture(scope="module")
def built_lib():
    from rendu_gb300 import build

    return build.build()


@pytest.mark.parametrize("compiler,std,ext", [("gcc", "-std=c11", "c"), ("g++", "-std=c++17", "cpp")])
def test_header_compiles_links_and_reports_status(built_lib, tmp_path, compiler, std, ext):
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not available")
    src = tmp_path / f"abi_check.{ext}"
    src.write_text(PROGRAM)
    exe = tmp_path / f"abi_check_{ext}"
    libdir = os.path.dirname(built_lib)
    libname = os.path.basename(built_lib)[3:-3]  # lib<name>.so -> <name>
    subprocess.run([compiler, std, "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", str(src), "-o",
                    str(exe), f"-L{libdir}", f"-l{libname}", f"-Wl,-rpath,{libdir}"], check=True, capture_output=True,
                   text=True)
    import torch

    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    if not torch.cuda.is_available():
        assert out.stdout.startswith("no-device")
