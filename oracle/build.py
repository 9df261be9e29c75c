"""Build recipe for the oracle (test infrastructure only).

- ``liboracle.so``: the CPU restatement in ``bsfit_oracle.cpp``, built on
  every machine that runs the tests, the smoke check or the benchmark.
- ``liboracle_fma.so``: the same source built with FMA contraction, the
  second FP64 build against which the parity tests measure the method's own
  reproducibility floor.
- ``_ref/libref_f32.so`` / ``_ref/libref_f64.so``: the reference's own CPU
  fitter compiled from its sources by ``build_ref.sh``, only where the reference
  sources exist; elsewhere the restatement alone is the oracle.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


def reference_root():
    """The reference project's root, from the BSFIT_REFERENCE_ROOT environment
    variable (no default: where it is unset, the reference is not built and the
    restatement alone, pinned by the committed golden fixtures, is the oracle)."""
    return os.environ.get("BSFIT_REFERENCE_ROOT") or None


def build_oracle(force=False):
    src = os.path.join(HERE, "bsfit_oracle.cpp")
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC",
           "-o", ORACLE_SO, src]
    subprocess.run(cmd, check=True)
    return ORACLE_SO


ORACLE_FMA_SO = os.path.join(HERE, "liboracle_fma.so")


def _fma_flags():
    """Flags that make g++ contract a * b + c into fused multiply-adds: none
    beyond -ffp-contract=fast on aarch64 (FMA is part of the base ISA), -mfma on
    x86-64 where the CPU has it; None where it has not."""
    import platform
    m = platform.machine().lower()
    if m in ("aarch64", "arm64"):
        return []
    if m in ("x86_64", "amd64"):
        try:
            with open("/proc/cpuinfo") as f:
                if " fma" in f.read():
                    return ["-mfma"]
        except OSError:
            pass
    return None


def build_oracle_fma(force=False):
    """The same restatement built with FMA contraction: a second, equally valid
    FP64 build of the reference method, whose results differ from the
    uncontracted build only by rounding. How often the two agree within the
    parity tolerances is the reproducibility floor of the method itself.
    Returns None where the CPU has no FMA."""
    flags = _fma_flags()
    if flags is None:
        return None
    src = os.path.join(HERE, "bsfit_oracle.cpp")
    if (not force and os.path.exists(ORACLE_FMA_SO)
            and os.path.getmtime(ORACLE_FMA_SO) >= os.path.getmtime(src)):
        return ORACLE_FMA_SO
    cmd = ["g++", "-O2", "-ffp-contract=fast", *flags, "-fopenmp", "-shared", "-fPIC",
           "-o", ORACLE_FMA_SO, src]
    subprocess.run(cmd, check=True)
    return ORACLE_FMA_SO


def build_reference(force=False, root=None):
    """Compile the reference CPU fitter from its sources under ``root`` (or
    BSFIT_REFERENCE_ROOT). Outputs already built are kept unless ``force``."""
    done = all(os.path.exists(os.path.join(REF_DIR, f))
               for f in ("libref_f32.so", "libref_f64.so", "ref_emccd.ptx"))
    if not force and done:
        return REF_DIR
    root = root or reference_root()
    if not root:
        return None
    src = os.path.join(root, "MultiD_bspline", "visual code", "CPUmleFit_LM", "CPUmleFit_LM.cpp")
    if not os.path.exists(src):
        return None
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), root], check=True)
    return REF_DIR


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_oracle_fma(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
