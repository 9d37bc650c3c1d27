"""CPU tests of the C-ABI library: it builds, loads, exports every symbol
include/ocean.h declares, and its host-only entry points (noise, FFT tables,
argument validation) behave -- no device call is made."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "ocean.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*OCEAN_API\s+(?:const\s+)?\w+\s*\*?\s*(ocean_\w+)\s*\(", src, flags=re.M)))


def test_exports_every_declared_symbol(ocean_lib):
    names = _declared_functions()
    assert len(names) >= 15
    lib = ocean_lib.load()
    for n in names:
        assert hasattr(lib, n), f"missing export {n}"
    assert sorted(ocean_lib.EXPORTS) == names


def test_only_c_abi_exported(ocean_lib):
    """Symbols are hidden by default: the library exports the C ABI only."""
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", ocean_lib.LIB_PATH], capture_output=True, text=True).stdout
    syms = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert syms and all(s.startswith("ocean_") for s in syms), syms


def test_noise_matches_oracle_bit_exact(ocean_lib, oracle_mod):
    for seed, N in [(0, 32), (1, 64), (123456789, 128)]:
        a = ocean_lib.fill_noise(seed, N)
        b = oracle_mod.noise(seed, N)
        assert np.array_equal(a, b)


def test_bit_reversed_indices(ocean_lib, oracle_mod):
    for N in (2, 32, 256, 2048, 65536):
        assert np.array_equal(ocean_lib.bit_reversed_indices(N), oracle_mod.bit_reversed(N))


def test_butterfly_table(ocean_lib, oracle_mod):
    for N in (32, 256, 1024):
        a = ocean_lib.butterfly_table(N).astype(np.float64)
        b = oracle_mod.twiddle_table(N)
        assert np.array_equal(a[..., 2:], b[..., 2:])
        assert np.abs(a[..., :2] - b[..., :2]).max() < 1e-7


@pytest.mark.parametrize("N", [0, 16, 48, 4096, -32])
def test_create_rejects_bad_n(ocean_lib, N):
    p = ocean_lib.Params(N=N)
    with pytest.raises(ocean_lib.OceanError) as e:
        ocean_lib.Ocean(p, seed=0)
    assert e.value.code == ocean_lib.OCEAN_ERR_INVALID
    assert "power of two" in str(e.value)


@pytest.mark.parametrize("field,val", [("L", 0.0), ("L", float("nan")), ("wind_speed", 0.0),
                                       ("amplitude", -1.0), ("wind_dir_x", float("inf"))])
def test_create_rejects_bad_params(ocean_lib, field, val):
    p = ocean_lib.Params(N=256)
    setattr(p, field, val)
    with pytest.raises(ocean_lib.OceanError) as e:
        ocean_lib.Ocean(p, seed=0)
    assert e.value.code == ocean_lib.OCEAN_ERR_INVALID


def test_zero_wind_direction_rejected(ocean_lib):
    p = ocean_lib.Params(N=256, wind_dir_x=0.0, wind_dir_y=0.0)
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.Ocean(p, seed=0)


def test_null_arguments(ocean_lib):
    lib = ocean_lib.load()
    assert lib.ocean_create(None, None, None) == ocean_lib.OCEAN_ERR_INVALID
    assert lib.ocean_update(None, 0.0, None, None) == ocean_lib.OCEAN_ERR_INVALID
    assert b"NULL" in lib.ocean_last_error()
    assert lib.ocean_fill_noise(0, 32, None) == ocean_lib.OCEAN_ERR_INVALID
    lib.ocean_destroy(None)


def test_header_is_c99_and_links(ocean_lib, tmp_path):
    """include/ocean.h compiles as strict C99 with warnings as errors, and a C
    program taking the address of every declared entry point links against
    the library (what a C host's binding would do)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = _declared_functions()
    src = tmp_path / "abi.c"
    src.write_text('#include "ocean.h"\n#include <stdio.h>\n'
                   "typedef void (*fn)(void);\n"
                   "static const fn table[] = {\n" + ",\n".join(f"    (fn){n}" for n in names) + "\n};\n"
                   "int main(void)\n{\n"
                   "    printf(\"%d %u\\n\", ocean_version(), (unsigned)(sizeof table / sizeof table[0]));\n"
                   "    return 0;\n}\n")
    lib_dir = os.path.dirname(ocean_lib.LIB_PATH)
    exe = tmp_path / "abi"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-Wno-pedantic", "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", lib_dir, "-locean_gb300",
                        f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["100", str(len(names))]
