"""Build helpers for the oracle libraries (test infrastructure).

``build_oracle()`` compiles ``pcisph_oracle.cpp`` into ``_build/libpcisph_oracle.so``;
``build_reference()`` runs ``build_ref.sh`` when the reference sources exist
(they do not on machines that only receive this repository's files).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libpcisph_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpcisph_ref.so")
# the reference checkout: $PCISPH_REFERENCE_DIR, else a checkout named "reference" beside this repository
REFERENCE_ROOT = os.environ.get("PCISPH_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                         "reference")

CXXFLAGS = ["-std=c++17", "-O3", "-fwrapv", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "pcisph_oracle.cpp")
    if force or _stale(ORACLE_SO, [src]):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        tmp = ORACLE_SO + ".tmp"
        subprocess.run(["g++", *CXXFLAGS, "-o", tmp, src], check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "PCISPH", "data", "kernels", "pcisph.cl"))


def build_reference(force=False):
    """Compile the reference kernels if their sources are present; returns the path or None."""
    if not reference_available():
        return REF_SO if os.path.exists(REF_SO) else None
    deps = [os.path.join(HERE, "build_ref.sh"), os.path.join(HERE, "ref_shim", "cl_shim.h"),
            os.path.join(HERE, "ref_shim", "ref_driver.cpp"), os.path.join(HERE, "ref_shim", "scene_shim.cpp"),
            os.path.join(HERE, "ref_shim", "scene_entry.cpp")]
    scene_so = os.path.join(os.path.dirname(REF_SO), "libpcisph_ref_scene.so")
    if force or _stale(REF_SO, deps) or _stale(scene_so, deps):
        subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT], check=True,
                       stdout=subprocess.DEVNULL)
    return REF_SO
