"""Build recipe for the reference-shader harness (test infrastructure only).

Where the reference sources are present, compiles the reference's own compute
shaders (src/shader/{tilde_h0_k,tilde_h0_t,twiddle_factors,butterfly,inversion,
normal_map}_cs.glsl) and its reverse_bits() (src/main.cpp:29-64, copied at
build time into oracle/_ref/ref_reverse_bits.inc, never into the repository)
together with oracle/ref_glsl/ into oracle/_ref/libref_glsl.so.

The rest of the reference (src/main.cpp as a whole) needs OpenGL, GLFW, ImGui
and the un-vendored dwSampleFramework and is not built.  The GPU machine has no
reference sources, so this library exists only where the golden fixtures are
generated (tests/golden/make_golden.py).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: OCEAN_REFERENCE_DIR, else a `reference` directory
# beside this repository's root.
REF = os.environ.get("OCEAN_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_glsl.so")
SHADERS = ["tilde_h0_k_cs.glsl", "tilde_h0_t_cs.glsl", "twiddle_factors_cs.glsl", "butterfly_cs.glsl",
           "inversion_cs.glsl", "normal_map_cs.glsl", "atmosphere.glsl", "sky_envmap_fs.glsl"]


def available() -> bool:
    return all(os.path.exists(os.path.join(REF, "src", "shader", s)) for s in SHADERS) and \
        os.path.exists(os.path.join(REF, "src", "main.cpp"))


def _extract_reverse_bits() -> str:
    with open(os.path.join(REF, "src", "main.cpp")) as fh:
        lines = fh.read().split("\n")
    seg = lines[28:64]  # main.cpp lines 29-64
    if not seg[0].startswith("const unsigned char g_bit_rev_table[]") or \
            not any(l.startswith("unsigned long reverse_bits(") for l in seg) or seg[-1] != "}":
        raise RuntimeError("main.cpp:29-64 is not the reverse_bits block this recipe expects")
    os.makedirs(OUT, exist_ok=True)
    path = os.path.join(OUT, "ref_reverse_bits.inc")
    with open(path, "w") as fh:
        fh.write("\n".join(seg) + "\n")
    return path


def _rewrite_atmosphere() -> str:
    """oracle/_ref/atmosphere.glsl: the reference's file with its `out vec3`
    parameters (SkyRadiance, InScattering) as C++ references, so that
    sky_envmap_fs.glsl's #include <atmosphere.glsl> compiles as C++."""
    with open(os.path.join(REF, "src", "shader", "atmosphere.glsl")) as fh:
        src = fh.read()
    n = src.count("out vec3 ")
    if n != 2:
        raise RuntimeError("atmosphere.glsl does not have the two `out vec3` parameters this recipe expects")
    os.makedirs(OUT, exist_ok=True)
    path = os.path.join(OUT, "atmosphere.glsl")
    with open(path, "w") as fh:
        fh.write(src.replace("out vec3 ", "vec3& "))
    return path


def build(force: bool = False, quiet: bool = True) -> str:
    if not available():
        raise RuntimeError(f"reference sources not found under {REF}")
    src = os.path.join(HERE, "ref_glsl", "ref_shaders.cpp")
    deps = [src] + [os.path.join(HERE, "ref_glsl", f) for f in ("glsl_shim.hpp", "glsl_begin.hpp", "glsl_end.hpp")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    _extract_reverse_bits()
    _rewrite_atmosphere()
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++20", "-O2", "-fPIC", "-shared", "-fopenmp", "-fsingle-precision-constant",
           "-ffp-contract=off", "-w", "-I", OUT, "-I", os.path.join(HERE, "ref_glsl"),
           "-I", os.path.join(REF, "src", "shader"), "-o", LIB + ".tmp", src]
    if not quiet:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_if_available() -> str | None:
    if not available():
        return None
    return build()


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, quiet=False))
