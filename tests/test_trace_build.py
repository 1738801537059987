"""The NVTX ranges of the C-ABI operations (VSL_RANGE in csrc/vsl_internal.h): a translation
unit using the macro compiles both ways, as a no-op statement by default and as an NVTX
push/pop pair with -DVSL_NVTX.  Host compile only (nvcc, no GPU); skipped without nvcc."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "2018_7_vesicle_gb300", "csrc")
UNIT = """#include "vsl_internal.h"
int traced(int x)
{
    VSL_RANGE(__func__);
    return x + 1;
}
"""


@pytest.mark.parametrize("flags", [[], ["-DVSL_NVTX"]])
def test_range_macro_compiles(tmp_path, flags):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    src = tmp_path / "traced.cu"
    src.write_text(UNIT)
    obj = tmp_path / "traced.o"
    r = subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I" + CSRC, *flags, "-c",
                        str(src), "-o", str(obj)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", "-u", str(obj)], capture_output=True, text=True).stdout
    # with the flag the range loader references dlopen; without it nothing of NVTX remains
    assert ("dlopen" in syms) == bool(flags)
