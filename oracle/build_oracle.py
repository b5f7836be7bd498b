"""CHECKER INFRASTRUCTURE (oracle): build the CPU checkers.

* oracle/_build/libdisco_port.so -- the plain-C restatement (oracle/port),
  compiled with -ffp-contract=off so x86 and Arm hosts round like the
  reference build (no fused multiply-add).
* oracle/_ref/<config>/disco_ref -- the reference itself, compiled from its
  unmodified sources by oracle/ref/Makefile, only where those sources exist:
  the directory named by the environment variable DISCO_REFERENCE, else the
  copy oracle/stage_reference.py leaves in baseline/_ref/src (git-ignored).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PORT_SRC = os.path.join(HERE, "port", "disco_port.c")
PORT_LIB = os.path.join(HERE, "_build", "libdisco_port.so")
REF_CONFIGS = ["configs/cfg1_vortex", "configs/cfg2_mhd_disk"]


def build_port(force: bool = False) -> str:
    hdrs = [os.path.join(ROOT, "include", "disco_gpu.h"),
            os.path.join(ROOT, "disco_gb300", "csrc", "plugins", "ic_vortex_gauss.h"),
            os.path.join(ROOT, "disco_gb300", "csrc", "plugins", "ic_disks.h"), PORT_SRC]
    if (not force and os.path.exists(PORT_LIB)
            and os.path.getmtime(PORT_LIB) >= max(os.path.getmtime(h) for h in hdrs)):
        return PORT_LIB
    os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
    tmp = PORT_LIB + ".tmp"
    subprocess.run(["gcc", "-std=gnu11", "-O3", "-fPIC", "-shared", "-ffp-contract=off",
                    f"-I{os.path.join(ROOT, 'include')}", PORT_SRC, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, PORT_LIB)
    return PORT_LIB


STAGED = os.path.join(ROOT, "baseline", "_ref", "src")


def reference_dir() -> str | None:
    """The reference source tree: $DISCO_REFERENCE, else the staged copy in
    baseline/_ref/src, else None."""
    env = os.environ.get("DISCO_REFERENCE")
    if env and os.path.isfile(os.path.join(env, "paul.h")):
        return env
    if os.path.isfile(os.path.join(STAGED, "paul.h")):
        return STAGED
    return None


def build_ref(reference: str | None = None, configs=None) -> list[str]:
    reference = reference or reference_dir()
    if not reference:
        return []
    out = []
    for cfg in configs or REF_CONFIGS:
        subprocess.run(["make", "-s", "-f", "oracle/ref/Makefile", f"CFG={cfg}", f"REF={reference}"],
                       cwd=ROOT, check=True)
        out.append(os.path.join(HERE, "_ref", os.path.basename(cfg), "disco_ref"))
    return out


def build_all() -> None:
    build_port()
    build_ref()


if __name__ == "__main__":
    build_all()
