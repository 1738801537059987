"""Build recipe for the oracle (TEST INFRASTRUCTURE ONLY).

* ``lib/libvsl_oracle.so`` from ``vsl_oracle.c`` (the C restatement), always;
* ``_ref/libvsl_ref.so`` from the reference's own kernel sources via ``ref/Makefile``, only
  where the reference checkout is present (it is read in place, never copied).

Both are built for the machine this runs on (x86 here, Arm on the GPU host).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout is read in place.  VSL_REFERENCE names its root; when it is unset
# the recipes look at the development container's read-only mount.
DEFAULT_REFERENCE = "/root/reference"
VESICLE = os.path.join("src", "7_0_paper", "2_0_Vesicle")


def reference_root() -> str:
    return os.environ.get("VSL_REFERENCE", DEFAULT_REFERENCE)


def reference_vesicle() -> str:
    """The vesicle project inside the reference checkout (the survey's V/)."""
    return os.path.join(reference_root(), VESICLE)


def reference_kernels() -> str:
    return os.path.join(reference_vesicle(), "CUDA_Code")


CFLAGS = ["-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-Wall"]


def build_port(force: bool = False) -> str:
    """lib/libvsl_oracle.so (pow from libm, as the reference) and
    lib/libvsl_oracle_crpow.so (integer powers rounded once, as the CUDA plain form)."""
    src = os.path.join(HERE, "vsl_oracle.c")
    deps = max(os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "vsl_oracle.h")))
    out = os.path.join(HERE, "lib", "libvsl_oracle.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    for path, extra in ((out, []), (os.path.join(HERE, "lib", "libvsl_oracle_crpow.so"), ["-DVSL_ORACLE_CR_POW"])):
        if force or not os.path.exists(path) or os.path.getmtime(path) < deps:
            subprocess.run(["gcc", *CFLAGS, *extra, "-o", path, src, "-lm"], check=True)
    return out


def build_ref() -> str | None:
    """Compile the reference kernels for the host; None when the checkout is absent."""
    kernels = reference_kernels()
    if not os.path.isdir(kernels):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"), f"REF={kernels}"], check=True)
    return os.path.join(HERE, "_ref", "libvsl_ref.so")


def build() -> None:
    build_port()
    build_ref()


if __name__ == "__main__":
    build()
