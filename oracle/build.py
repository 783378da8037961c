"""Build recipes of the CPU oracle (test infrastructure).

* ``build_oracle()``: ``oracle/liboracle.so`` from nr_oracle.cpp + sparse_lu.cpp (this
  project's restatement of the reference's CPU solver). Built with ``-ffp-contract=off``
  so x86 and Arm builds round alike.
* ``build_reference()``: the reference's OWN ``p3s/cpp/nr_klu.cpp`` (+ ``lean_lu.hpp``,
  ``finite.hpp``), compiled where it lies under the read-only reference checkout with the
  flags of its ``p3s/cpp/CMakeLists.txt:32-35`` (``-O3 -funroll-loops -ffast-math``,
  OpenMP), pybind11, and the project's KLU-API shim (klu_shim/) standing in for
  SuiteSparse KLU. Output goes to ``oracle/_ref/`` only. Needs the reference checkout
  (``$P3S_REFERENCE``, default ``../reference`` beside the repository) and pybind11, so it is
  built only where both exist.
"""

from __future__ import annotations

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: P3S_REFERENCE, else the checkout beside this repository's parent
REFERENCE = os.environ.get("P3S_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
REF_CPP = os.path.join(REFERENCE, "p3s", "cpp")


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")


def oracle_cmd():
    out = os.path.join(HERE, "liboracle.so")
    return out, [
        "g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC",
        os.path.join(HERE, "nr_oracle.cpp"), os.path.join(HERE, "sparse_lu.cpp"), "-o", out,
    ]


def build_oracle(force: bool = False) -> str:
    out, cmd = oracle_cmd()
    srcs = [os.path.join(HERE, f) for f in ("nr_oracle.cpp", "sparse_lu.cpp", "sparse_lu.h")]
    if force or not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(s) for s in srcs):
        _run(cmd)
    return out


def reference_available() -> bool:
    if not os.path.exists(os.path.join(REF_CPP, "nr_klu.cpp")):
        return False
    try:
        import pybind11  # noqa: F401
    except ImportError:
        return False
    return True


# Two builds of the same reference sources: "fastmath" with the reference's own release
# flags, and "strict" (IEEE, no FMA contraction) against which the oracle restatement is
# expected to agree bit for bit.
# The strict build is renamed at compile time (-Dnr_klu=nr_klu_strict renames the module
# token of PYBIND11_MODULE; a distinct PYBIND11_BUILD_ABI keeps its type registry apart)
# so that both can be imported into one process.
VARIANTS = {
    "fastmath": ["-O3", "-funroll-loops", "-ffast-math"],
    "strict": ["-O2", "-ffp-contract=off", "-Dnr_klu=nr_klu_strict", "-DPYBIND11_BUILD_ABI=\"_p3s_strict\""],
}
MODULE = {"fastmath": "nr_klu", "strict": "nr_klu_strict"}


def reference_cmd(variant: str = "fastmath"):
    import pybind11

    ext = sysconfig.get_config_var("EXT_SUFFIX")
    out = os.path.join(HERE, "_ref", variant, MODULE[variant] + ext)
    inc = [f"-I{pybind11.get_include()}", f"-I{sysconfig.get_paths()['include']}"]
    return out, [
        "g++", *VARIANTS[variant], "-fopenmp", "-std=c++17", "-shared", "-fPIC", *inc,
        f"-I{os.path.join(HERE, 'klu_shim')}", f"-I{REF_CPP}",
        os.path.join(REF_CPP, "nr_klu.cpp"), os.path.join(HERE, "klu_shim", "klu_shim.cpp"),
        os.path.join(HERE, "sparse_lu.cpp"), "-o", out,
    ]


def reference_jobs(force: bool = False):
    """(output, command) of every reference build still to do."""
    if not reference_available():
        return []
    jobs = []
    for v in VARIANTS:
        os.makedirs(os.path.join(HERE, "_ref", v), exist_ok=True)
        out, cmd = reference_cmd(v)
        if force or not os.path.exists(out):
            jobs.append((out, cmd))
    return jobs


def build_reference(force: bool = False) -> list[str]:
    outs = []
    for out, cmd in reference_jobs(force):
        _run(cmd)
        outs.append(out)
    return outs


def load_reference(variant: str = "fastmath"):
    """The reference's own nr_klu module built by build_reference(), or None."""
    import importlib.util

    d = os.path.join(HERE, "_ref", variant)
    if not os.path.isdir(d):
        return None
    name = MODULE[variant]
    files = [f for f in os.listdir(d) if f.startswith(name + ".") and f.endswith(".so")]
    if not files:
        return None
    key = f"_ref_{name}"
    if key in sys.modules:
        return sys.modules[key]
    spec = importlib.util.spec_from_file_location(name, os.path.join(d, files[0]))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.modules[key] = mod
    return mod


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_reference(force=True))
