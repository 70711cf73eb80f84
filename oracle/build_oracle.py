"""Build recipe for the test oracle — TEST INFRASTRUCTURE ONLY.

* ``build_oracle()`` compiles ``oracle/lof_oracle.c`` (our plain-C restatement)
  with gcc into ``oracle/_build/liblof_oracle.so``. It builds on any host
  (x86_64 here, aarch64 on the GPU machine).
* ``build_ref()`` compiles ``oracle/ref_shim.cpp`` against the reference's own
  headers where they lie (``$LOFGB_REFERENCE/src``, default
  ``/root/reference/src``) into ``oracle/_ref/libref_shim.so``. It is skipped
  when the reference checkout is absent. Only tests/golden/make_golden.py and
  the optional oracle-vs-reference test use it.

Both use ``-ffp-contract=off`` so the compiler never fuses the two-sum and
scale arithmetic into FMAs (GCC contracts by default on aarch64).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_OUT_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liblof_oracle.so")
REF_SO = os.path.join(REF_OUT_DIR, "libref_shim.so")


def reference_src_dir() -> str:
    return os.path.join(os.environ.get("LOFGB_REFERENCE", "/root/reference"), "src")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "lof_oracle.c"), os.path.join(HERE, "lof_oracle.h"),
            os.path.join(HERE, "..", "include", "lofgb.h")]
    if force or _stale(ORACLE_SO, srcs):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = ORACLE_SO + f".tmp{os.getpid()}"
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas", srcs[0], "-o", tmp, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force: bool = False) -> str | None:
    src_dir = reference_src_dir()
    if not os.path.exists(os.path.join(src_dir, "lo_float.h")):
        return None
    shim = os.path.join(HERE, "ref_shim.cpp")
    if not (force or _stale(REF_SO, [shim])):
        return REF_SO
    try:
        import torch.utils.cpp_extension as ce  # c10/util/Half.h for the half path
        torch_inc = ce.include_paths()
    except Exception:  # pragma: no cover - torch is always present here
        torch_inc = []
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    os.makedirs(REF_OUT_DIR, exist_ok=True)
    tmp = REF_SO + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-DUSE_CUDA", "-frounding-math",
           "-ffp-contract=off", "-w", "-I" + src_dir, "-I" + os.path.join(cuda, "include"),
           "-I" + os.path.join(cuda, "include", "cccl")]
    cmd += ["-I" + p for p in torch_inc]
    cmd += [shim, "-o", tmp]
    _run(cmd)
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
