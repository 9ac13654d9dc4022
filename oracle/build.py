"""Build recipe for the CPU oracle (test infrastructure, not the product).

* ``oracle/liboracle.so``: the portable C restatement in ``oracle/goto.c``.
  Builds on x86-64 and aarch64 alike; ``-ffp-contract=off`` keeps every
  rounding where the source puts it (``fma()`` calls stay fused, plain ``a*b+c``
  stays two roundings), which is what makes it bit-identical to the
  reference microkernels.
* ``oracle/_ref/libref_ukr.so``: the reference's own vendored BLIS Haswell
  microkernels (``ukernels/bli_gemm_haswell_asm_d6x8.c`` and ``..._d4x12.c``),
  compiled unmodified from the reference checkout with a typedef-only
  ``blis.h`` stub. x86-64 only (the kernels are AVX2/FMA inline assembly) and
  only where the reference checkout exists; everywhere else it is skipped.

Where the checkout is: the directory named by ``--reference DIR`` (when run
as a script) or the ``MOMMS_REFERENCE_ROOT`` environment variable; unset, a
``reference`` directory beside the repository (``../reference`` from its
root) if one is there. With none of these the reference build is skipped.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO_ROOT = os.path.dirname(HERE)


def reference_root():
    """The reference checkout, or None (see the module docstring)."""
    env = os.environ.get("MOMMS_REFERENCE_ROOT")
    if env:
        return env
    sibling = os.path.join(os.path.dirname(REPO_ROOT), "reference")
    return sibling if os.path.isdir(sibling) else None


REF_KERNELS = [
    "ukernels/bli_gemm_haswell_asm_d6x8.c",
    "ukernels/bli_gemm_haswell_asm_d4x12.c",
]
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_ukr.so")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(verbose=False):
    src = os.path.join(HERE, "goto.c")
    if _newer(ORACLE_SO, [src, __file__]):
        return ORACLE_SO
    flags = ["-O3", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # hardware fma(); same results as the libm call
    cmd = ["gcc", *flags, src, "-o", ORACLE_SO + ".tmp", "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_ref(verbose=False, root=None):
    """Compile the reference's own microkernels; returns the path or None."""
    if platform.machine() not in ("x86_64", "AMD64"):
        return None
    root = root or reference_root()
    if not root:
        return None
    srcs = [os.path.join(root, s) for s in REF_KERNELS]
    if not all(os.path.exists(s) for s in srcs):
        return None
    if _newer(REF_SO, srcs + [__file__]):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    cmd = ["gcc", "-O2", "-mavx2", "-mfma", "-fPIC", "-shared",
           "-I", os.path.join(HERE, "ref_stub"), *srcs, "-o", REF_SO + ".tmp"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(REF_SO + ".tmp", REF_SO)
    return REF_SO


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=None, help="reference checkout (default: see module docstring)")
    args = ap.parse_args()
    print(build_oracle(verbose=True))
    print(build_ref(verbose=True, root=args.reference))
    sys.exit(0)
