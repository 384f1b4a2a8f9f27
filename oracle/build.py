"""Build recipe for the oracle (test infrastructure only).

- ``build_oracle()`` compiles the C restatement ``vt_oracle.c`` into ``oracle/_build/``.
- ``build_ref()`` compiles vtrace's own fragment shader, ``shaders/trace.frag`` from the
  reference source tree, as C++: the shader text minus its ``#version``/``#extension`` lines is
  piped to g++ with ``glsl_compat.hpp`` force-included, and linked with ``ref_harness.cpp`` into
  ``oracle/_ref/``.  Two builds: ``select`` (b2f-multiply read as a select, the canonical reading)
  and ``ieee`` (literal IEEE product).  Skipped when the reference tree is absent.

Both use -ffp-contract=off so that each float operator is one IEEE binary32 operation.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference source tree: VTRACE_REFERENCE when set, else where this build's recipe finds it in
# the build container.  It is read here only (the GPU machine has no copy); tests that need it ask
# reference_root() and skip when it returns None.
_DEFAULT_REFERENCE = "/root/reference"


def reference_root():
    """The reference source tree's root, or None where it is absent."""
    root = os.environ.get("VTRACE_REFERENCE") or _DEFAULT_REFERENCE
    return root if os.path.isdir(root) else None


REFERENCE = reference_root()
SHADER = os.path.join(REFERENCE, "shaders", "trace.frag") if REFERENCE else ""

ORACLE_SO = os.path.join(BUILD, "libvt_oracle.so")


def ref_so(variant="select"):
    return os.path.join(REF_OUT, "libvt_tracefrag_%s.so" % variant)


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "vt_oracle.c")
    hdr = os.path.join(HERE, "vt_oracle.h")
    if not force and _newer(ORACLE_SO, [src, hdr, __file__]):
        return ORACLE_SO
    os.makedirs(BUILD, exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(
        ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
         "-pthread", src, "-o", tmp, "-lm"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force=False):
    """Returns the list of built libraries, or [] when the reference tree is absent."""
    if not SHADER or not os.path.exists(SHADER):
        return []
    compat = os.path.join(HERE, "glsl_compat.hpp")
    harness = os.path.join(HERE, "ref_harness.cpp")
    os.makedirs(REF_OUT, exist_ok=True)
    built = []
    for variant, flag in (("select", "1"), ("ieee", "0")):
        out = ref_so(variant)
        if not force and _newer(out, [SHADER, compat, harness, __file__]):
            built.append(out)
            continue
        obj = os.path.join(REF_OUT, "trace_frag_%s.o" % variant)
        common = ["g++", "-std=gnu++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                  "-w", "-DVT_B2F_SELECT=" + flag, "-I", HERE]
        sed = subprocess.run(["sed", "/^#version/d;/^#extension/d", SHADER], check=True,
                             stdout=subprocess.PIPE)
        subprocess.run(common + ["-include", compat, "-x", "c++", "-c", "-", "-o", obj],
                       input=sed.stdout, check=True)
        tmp = out + ".tmp%d" % os.getpid()
        subprocess.check_call(common + ["-shared", harness, obj, "-o", tmp])
        os.replace(tmp, out)
        os.remove(obj)
        built.append(out)
    return built


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
