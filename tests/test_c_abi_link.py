"""The public headers compile as C (C11, no C++) and a C program links
against libops_fft.so and calls the API: the binding a C caller of the
reference would use.  No kernel runs (plans on a machine without a GPU defer
their device set-up), so this is a CPU test."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "ops-fft_gb300")

C_SRC = r"""
#include <stdio.h>
#include <string.h>
#include "cann_ops_fft.h"
#include "aclfft_ext.h"
#include "aclfft_ops.h"

#define CHECK(cond) do { if (!(cond)) { printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond); return 1; } } while (0)

int main(void)
{
    aclfftHandle plan = NULL;
    size_t ws = 123;
    int v = 0, major = -1;
    float in[2 * 8], out[2 * 8];
    int i;

    CHECK(strcmp(aclfftGetErrorString(ACLFFT_SUCCESS), "Success") == 0);
    CHECK(aclfftGetVersion(&v) == ACLFFT_SUCCESS && v == ACLFFT_GB300_VERSION);
    CHECK(aclfftGetProperty(ACLFFT_MAJOR_VERSION, &major) == ACLFFT_SUCCESS && major == v / 10000);

    CHECK(aclfftCreate(&plan) == ACLFFT_SUCCESS);
    CHECK(aclfftMakePlan1d(plan, 3000, ACLFFT_R2C, 4096, ACLFFT_HORIZONTAL, &ws) == ACLFFT_SUCCESS);
    CHECK(aclfftGetSize(plan, &ws) == ACLFFT_SUCCESS);
    CHECK(aclfftMakePlan1d(plan, 3000, ACLFFT_R2C, 4096, ACLFFT_HORIZONTAL, &ws) == ACLFFT_INVALID_VALUE);
    CHECK(aclfftSetNormMode(plan, ACLFFT_NORM_BACKWARD) == ACLFFT_SUCCESS);
    CHECK(aclfftSetStream(plan, (cudaStream_t)0) == ACLFFT_SUCCESS);
    CHECK(aclfftDestroy(plan) == ACLFFT_SUCCESS);

    CHECK(aclfftPlan2d(&plan, 2, 64, 100, ACLFFT_C2R) == ACLFFT_SUCCESS);
    CHECK(aclfftDestroy(plan) == ACLFFT_SUCCESS);
    CHECK(aclfftPlan3d(&plan, 8, 8, 8, ACLFFT_C2C) == ACLFFT_SUCCESS);
    CHECK(aclfftDestroy(plan) == ACLFFT_SUCCESS);
    plan = NULL;
    CHECK(aclfftPlan3d(&plan, 8, 8, 8, (aclfftType)0x2b) == ACLFFT_INVALID_TYPE && plan == NULL);
    CHECK(aclfftGetSize1d(NULL, 64, ACLFFT_C2C, 1, &ws) == ACLFFT_INVALID_VALUE);

    /* per-operator entries: argument checks return aclError codes */
    CHECK(aclfftFft1DC2C(NULL, NULL, 64, -1, 1, 0, NULL) == ACL_ERROR_INVALID_PARAM);

    /* the host butterfly hook: radix 8 of a delta is all ones */
    for (i = 0; i < 16; ++i) in[i] = 0.f;
    in[0] = 1.f;
    CHECK(aclfftDebugButterfly(8, in, out) == ACLFFT_SUCCESS);
    for (i = 0; i < 8; ++i) CHECK(out[2 * i] == 1.f && out[2 * i + 1] == 0.f);
    printf("ok\n");
    return 0;
}
"""


def test_c_program_compiles_links_and_runs(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = os.path.join(LIBDIR, "libops_fft.so")
    assert os.path.exists(lib), "build the library first (ops-fft_gb300/build.py)"
    cuda_inc = None
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "include", "cuda_runtime_api.h")):
            cuda_inc = os.path.join(c, "include")
            break
    if cuda_inc is None:
        pytest.skip("CUDA headers not found")
    src = tmp_path / "app.c"
    src.write_text(C_SRC)
    exe = tmp_path / "app"
    cmd = [cc, "-std=c11", "-Wall", "-Werror", "-pedantic", str(src), "-I", os.path.join(ROOT, "include"),
           "-I", cuda_inc, "-L", LIBDIR, "-lops_fft", "-Wl,-rpath," + LIBDIR, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, OPS_FFT_LOG="0")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.stdout[-2000:], r.stderr[-2000:])
