"""Build recipes for the CPU oracle (test infrastructure).

- ``build_oracle()`` compiles oracle/proj_oracle.cpp, the restatement of the
  reference arithmetic, into oracle/_build/libproj_oracle.so.
- ``build_ref()`` compiles the two standalone pieces of the so3g reference
  (include/so_linterp.h and src/healpix_bare.c, read in place from the
  reference checkout) plus oracle/ref_parts.cpp into
  oracle/_ref/libref_parts.so.  It returns None where the reference
  checkout is absent.

Both use ``-ffp-contract=off`` so that no multiply-add is fused: the float64
results then equal those of an x86-64 build of the reference on any host.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# The so3g reference checkout: $SO3G_REFERENCE, else a checkout named
# "reference" beside this repository's directory (absent on machines that
# only run the tests; build_ref() then builds nothing).
REFERENCE = os.environ.get(
    "SO3G_REFERENCE",
    os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))

ORACLE_SO = os.path.join(HERE, "_build", "libproj_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_parts.so")
REF_ENGINE_SO = os.path.join(HERE, "_ref", "libref_engine.so")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def oracle_cmd():
    src = os.path.join(HERE, "proj_oracle.cpp")
    return ["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
            "-std=c++17", src, "-o", ORACLE_SO]


def build_oracle(force=False):
    srcs = [os.path.join(HERE, f) for f in ("proj_oracle.cpp", "proj_oracle.h")]
    srcs.append(os.path.join(HERE, "..", "include", "so3g_gb300.h"))
    if force or _stale(ORACLE_SO, srcs):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        _run(oracle_cmd())
    return ORACLE_SO


def build_ref(force=False):
    hp_c = os.path.join(REFERENCE, "src", "healpix_bare.c")
    inc = os.path.join(REFERENCE, "include")
    if not (os.path.exists(hp_c) and os.path.exists(os.path.join(inc, "so_linterp.h"))):
        return None
    wrapper = os.path.join(HERE, "ref_parts.cpp")
    if force or _stale(REF_SO, [wrapper, hp_c]):
        out = os.path.dirname(REF_SO)
        os.makedirs(out, exist_ok=True)
        hp_o = os.path.join(out, "healpix_bare.o")
        _run(["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-c", "-I", inc,
              hp_c, "-o", hp_o])
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", inc,
              wrapper, hp_o, "-o", REF_SO])
    return REF_SO


def ref_sources_present():
    return os.path.exists(os.path.join(REFERENCE, "src", "Projection.cxx"))


def build_ref_engine(force=False):
    """Compiles the reference's src/Projection.cxx, read in place from the
    reference checkout, with the stand-in headers of oracle/refstub and the
    wrapper oracle/ref_engine.cpp into oracle/_ref/libref_engine.so (a
    library loaded into Python with ctypes.PyDLL).  Returns None where the
    reference checkout is absent."""
    if not ref_sources_present():
        return None
    import sysconfig
    import numpy
    stub = os.path.join(HERE, "refstub")
    srcs = [os.path.join(HERE, "ref_engine.cpp"), os.path.join(HERE, "ref_numpy.cpp")]
    deps = srcs + [os.path.join(REFERENCE, "src", "Projection.cxx")] + [
        os.path.join(d, f) for d, _, fs in os.walk(stub) for f in fs]
    if force or _stale(REF_ENGINE_SO, deps):
        os.makedirs(os.path.dirname(REF_ENGINE_SO), exist_ok=True)
        tmp = REF_ENGINE_SO + ".tmp"
        _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
              "-DNDEBUG", "-I", stub, "-I", os.path.join(REFERENCE, "include"),
              "-I", os.path.join(REFERENCE, "src"), "-I", sysconfig.get_paths()["include"],
              "-I", numpy.get_include()] + srcs + ["-o", tmp])
        os.replace(tmp, REF_ENGINE_SO)
    return REF_ENGINE_SO


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
    print(build_ref_engine())
