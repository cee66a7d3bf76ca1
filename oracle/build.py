"""Build recipes for the test oracle (test infrastructure, not the product).

* ``build_oracle()`` compiles the CPU restatement in ``oracle/*.c`` into
  ``oracle/_build/liboracle.so`` with gcc.  It runs on any machine.
* ``build_ref()`` compiles the reference's own C sources, where they lie in
  the read-only reference tree, into ``oracle/_ref/``: ``libmpm_ref.so`` (the
  reference's libmpm), one plugin ``.so`` per material and boundary condition,
  ``libref_harness.so`` (the driver set-up of src/main.c:415-835 without
  libconfuse, linked with the reference's src/writer.c) and the ``material_<name>`` executables of tests/test_material.c.
  It needs the reference tree and is skipped where it is absent.

Two deviations are applied while compiling, never by copying source into this
repository:
  * materialsrc/g_nonlocal_mu2.c:154 declares ``lambda`` without initialising
    it before use at :169-171; the source is piped through ``sed`` to give it
    the value ``K - 2.0 * G / 3.0`` that :257 uses.
  * CXSparse is absent, so the nonlocal plugins link ``oracle/ref/cs_shim.c``.
All of it is compiled with ``-ffp-contract=off`` so that results do not depend
on whether the compiler fuses multiply-adds.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
BUILD_OUT = os.path.join(HERE, "_build")
DEFAULT_REFERENCE = "/root/reference"

CFLAGS = ["-O2", "-std=gnu99", "-fPIC", "-ffp-contract=off", "-w"]
# The reference's own release flags (CMakeLists.txt:4), for timing it only:
# with contraction left on, its results are not the bit-exact golden source.
PERF_CFLAGS = ["-O3", "-march=native", "-std=gnu99", "-fPIC", "-w"]
PERF_OUT = os.path.join(REF_OUT, "perf")

LIBMPM_SOURCES = ["element.c", "interpolate.c", "loading.c", "map.c", "material.c",
                  "particle.c", "process_usl.c", "rtsafe.c", "tensor.c"]
KAT_MATERIALS = ["isolin", "g_local_mu2", "dp_ri_mt", "g_local_mu2_plane_strain", "g_local_mu2_true_2d",
                 "g_local_mu2_reverse"]
# g_local_mu2_ext needs the team's element lists and barrier, which
# tests/test_material.c does not set up: plugin only
LOCAL_MATERIALS = KAT_MATERIALS + ["g_local_mu2_ext"]
NONLOCAL_MATERIALS = ["g_nonlocal_mu2", "g_nonlocal", "g_nonlocal_avg", "g_nonlocal_bicgstab", "g_nonlocalxs71"]
BCS = ["box", "square_silo"]


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def reference_dir():
    return os.environ.get("MPM_REFERENCE_DIR", DEFAULT_REFERENCE)


def have_reference():
    return os.path.isfile(os.path.join(reference_dir(), "libmpm", "process_usl.c"))


def build_oracle(verbose=False):
    """Compile the CPU restatement into oracle/_build/liboracle.so."""
    os.makedirs(BUILD_OUT, exist_ok=True)
    out = os.path.join(BUILD_OUT, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("mpm_oracle.c", "banded.c")]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "mpm_oracle.h")])
    if os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
           "-Wall", "-Wextra", "-Wno-unused-parameter", "-o", out] + srcs + ["-lm", "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    _run(cmd)
    return out


def build_ref(verbose=False):
    """Compile the reference's own sources into oracle/_ref/.  Returns the
    output directory, or None when the reference tree is absent."""
    if not have_reference():
        return None
    ref = reference_dir()
    os.makedirs(REF_OUT, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "ref", "include"), "-I", os.path.join(ref, "libmpm")]
    rpath = ["-Wl,-rpath,$ORIGIN"]
    link_mpm = ["-L", REF_OUT, "-lmpm_ref"] + rpath

    def sh(cmd):
        if verbose:
            print(" ".join(cmd))
        _run(cmd)

    libmpm = os.path.join(REF_OUT, "libmpm_ref.so")
    sh(["gcc"] + CFLAGS + inc + ["-shared", "-o", libmpm]
       + [os.path.join(ref, "libmpm", s) for s in LIBMPM_SOURCES] + ["-lm", "-lpthread"])

    shim = os.path.join(HERE, "ref", "cs_shim.c")
    band = os.path.join(HERE, "banded.c")
    for mat in LOCAL_MATERIALS:
        sh(["gcc"] + CFLAGS + inc + ["-shared", "-o", os.path.join(REF_OUT, mat + ".so"),
                                     os.path.join(ref, "materialsrc", mat + ".c")] + link_mpm + ["-lm"])
    for mat in NONLOCAL_MATERIALS:
        src = os.path.join(ref, "materialsrc", mat + ".c")
        out = os.path.join(REF_OUT, mat + ".so")
        if mat == "g_nonlocal_mu2":
            # Give the uninitialised lambda (g_nonlocal_mu2.c:154) the value of :257.
            sed = subprocess.run(
                ["sed", "-e", r"s/^\(\s*\)double trD, lambda;/\1double trD, lambda = K - 2.0 * G \/ 3.0;/", src],
                capture_output=True, text=True, check=True)
            if "lambda = K - 2.0 * G / 3.0;" not in sed.stdout.split("calculate_bulk_granular_fluidity(job);")[0]:
                raise RuntimeError("lambda fix did not apply to %s" % src)
            cmd = (["gcc"] + CFLAGS + inc + ["-I", os.path.join(ref, "materialsrc"), "-shared", "-o", out,
                    "-x", "c", "-", "-x", "none", shim, band] + link_mpm + ["-lm"])
            if verbose:
                print(" ".join(cmd), "< (patched", src, ")")
            r = subprocess.run(cmd, input=sed.stdout, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(r.stderr)
        else:
            sh(["gcc"] + CFLAGS + inc + ["-shared", "-o", out, src, shim, band] + link_mpm + ["-lm"])
    for bc in BCS:
        sh(["gcc"] + CFLAGS + inc + ["-shared", "-o", os.path.join(REF_OUT, bc + ".so"),
                                     os.path.join(ref, "bcsrc", bc + ".c")] + link_mpm + ["-lm"])

    # the harness links the reference's own writer (src/writer.c) for golden frame and state text
    sh(["gcc"] + CFLAGS + inc + ["-I", os.path.join(ref, "src"), "-shared", "-o",
                                 os.path.join(REF_OUT, "libref_harness.so"),
                                 os.path.join(HERE, "ref", "ref_harness.c"), os.path.join(ref, "src", "writer.c")]
       + link_mpm + ["-ldl", "-lpthread", "-lm"])

    for mat in KAT_MATERIALS:
        sh(["gcc"] + CFLAGS + inc + ["-o", os.path.join(REF_OUT, "material_" + mat),
                                     os.path.join(ref, "tests", "test_material.c"),
                                     os.path.join(ref, "materialsrc", mat + ".c")] + link_mpm + ["-lm", "-lpthread"])
    return REF_OUT


def build_ref_perf(materials=("isolin", "g_local_mu2"), verbose=False):
    """Compile the reference's libmpm, the given local materials, the box and
    square_silo plugins and the harness with the reference's own release
    flags into oracle/_ref/perf/ (the timed CPU baseline).  Returns the
    directory, or None when the reference tree is absent."""
    if not have_reference():
        return None
    ref = reference_dir()
    os.makedirs(PERF_OUT, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "ref", "include"), "-I", os.path.join(ref, "libmpm")]
    link_mpm = ["-L", PERF_OUT, "-lmpm_ref"] + ["-Wl,-rpath,$ORIGIN"]

    def sh(cmd):
        if verbose:
            print(" ".join(cmd))
        _run(cmd)

    sh(["gcc"] + PERF_CFLAGS + inc + ["-shared", "-o", os.path.join(PERF_OUT, "libmpm_ref.so")]
       + [os.path.join(ref, "libmpm", f) for f in LIBMPM_SOURCES] + ["-lm", "-lpthread"])
    for mat in materials:
        sh(["gcc"] + PERF_CFLAGS + inc + ["-shared", "-o", os.path.join(PERF_OUT, mat + ".so"),
                                          os.path.join(ref, "materialsrc", mat + ".c")] + link_mpm + ["-lm"])
    for bc in BCS:
        sh(["gcc"] + PERF_CFLAGS + inc + ["-shared", "-o", os.path.join(PERF_OUT, bc + ".so"),
                                          os.path.join(ref, "bcsrc", bc + ".c")] + link_mpm + ["-lm"])
    sh(["gcc"] + PERF_CFLAGS + inc + ["-I", os.path.join(ref, "src"), "-shared", "-o",
                                      os.path.join(PERF_OUT, "libref_harness.so"),
                                      os.path.join(HERE, "ref", "ref_harness.c"), os.path.join(ref, "src", "writer.c")]
       + link_mpm + ["-ldl", "-lpthread", "-lm"])
    return PERF_OUT


if __name__ == "__main__":
    print(build_oracle(verbose=True) if "oracle" in sys.argv[1:] else build_ref(verbose=True))
