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


STRUCTS = ["ocean_params", "ocean_outputs", "ocean_grads", "ocean_grid_params", "ocean_shade_params",
           "ocean_sky_params", "ocean_tuning"]


def _c_layout(tmp_path, structs):
    """sizeof and every field's offsetof, as a C compiler lays out the
    structs of include/ocean.h: {struct: (size, {field: offset})}."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include "ocean.h"', "#include <stddef.h>", "#include <stdio.h>", "int main(void)", "{"]
    for name, fields in structs.items():
        lines.append(f'    printf("{name} .sizeof %zu\\n", sizeof({name}));')   # no field is named so
        for f in fields:
            lines.append(f'    printf("{name} {f} %zu\\n", offsetof({name}, {f}));')
    lines += ["    return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    res = {}
    for ln in filter(None, out):
        name, key, val = ln.split()
        entry = res.setdefault(name, [0, {}])
        if key == ".sizeof":
            entry[0] = int(val)
        else:
            entry[1][key] = int(val)
    return {k: (v[0], v[1]) for k, v in res.items()}


def test_ctypes_structs_match_the_header(ocean_lib, tmp_path):
    """Every ctypes structure of the binding has the C header's size, field
    names, field order and field offsets (a mismatch would pass arguments
    silently wrong)."""
    import ctypes
    structs = {n: [f[0] for f in getattr(ocean_lib, n)._fields_] for n in STRUCTS}
    c = _c_layout(tmp_path, structs)
    for n in STRUCTS:
        cls = getattr(ocean_lib, n)
        size, offs = c[n]
        assert ctypes.sizeof(cls) == size, n
        assert [getattr(cls, f).offset for f in structs[n]] == [offs[f] for f in structs[n]], n
        # the header declares no fields beyond these: the last one ends the struct
        last = structs[n][-1]
        assert offs[last] + ctypes.sizeof(dict(cls._fields_)[last]) <= size
        assert size - (offs[last] + ctypes.sizeof(dict(cls._fields_)[last])) < 8, n


def test_ctypes_stub_matches_the_binding(ocean_lib):
    """The minimal ctypes binding a maintainer copies (ctypes_stub.py) has the
    full binding's structures (same field names and types in the same order)
    and loads the library's per-frame entry points."""
    import ctypes_stub
    for n in ("ocean_params", "ocean_outputs"):
        assert getattr(ctypes_stub, n)._fields_ == getattr(ocean_lib, n)._fields_, n
    lib = ctypes_stub.load(ocean_lib.LIB_PATH)
    for name in ("ocean_create_seeded", "ocean_update", "ocean_destroy", "ocean_last_error"):
        assert hasattr(lib, name)


def _c_kind(t):
    """Canonical kind of a C parameter or return type of include/ocean.h."""
    t = " ".join(t.replace("const", " ").split())
    if "*" in t:
        return "ptr"
    return {"void": None, "int": "i32", "int32_t": "i32", "uint32_t": "u32", "int64_t": "i64",
            "uint64_t": "u64", "float": "f32", "double": "f64"}[t]


def _ctypes_kind(t):
    if t is None:
        return None
    if t in (C.c_void_p, C.c_char_p) or isinstance(t, type(C.POINTER(C.c_int))):
        return "ptr"
    for kind, ts in (("i32", (C.c_int, C.c_int32)), ("u32", (C.c_uint32,)), ("i64", (C.c_int64,)),
                     ("u64", (C.c_uint64,)), ("f32", (C.c_float,)), ("f64", (C.c_double,))):
        if t in ts:
            return kind
    raise AssertionError(f"unexpected ctypes type {t}")


def test_ctypes_signatures_match_the_header(ocean_lib):
    """Each entry point's ctypes argtypes and restype in the binding have the
    kinds (pointer, 32/64-bit integer, float, double) of its prototype in
    include/ocean.h.  A double passed where the C side expects an int would
    otherwise go through silently."""
    src = open(os.path.join(ROOT, "include", "ocean.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = re.findall(r"OCEAN_API\s+([\w\s\*]+?)\s*\b(ocean_\w+)\s*\(([^)]*)\)\s*;", src)
    assert len(protos) == len(_declared_functions())
    lib = ocean_lib.load()
    for ret, name, params in protos:
        params = " ".join(params.split())
        kinds = [] if params in ("", "void") else [
            _c_kind(re.sub(r"\b\w+$", "", p.strip()) if not p.strip().endswith("*") else p) for p in params.split(",")]
        fn = getattr(lib, name)
        if fn.argtypes is None:
            assert kinds == [], f"{name}: the binding sets no argtypes for {kinds}"
        else:
            assert [_ctypes_kind(t) for t in fn.argtypes] == kinds, name
        want = _c_kind(ret)
        got = _ctypes_kind(fn.restype)
        assert got == want, f"{name}: restype {got} vs {want}"


def test_grid_parameter_validation_before_any_device_call(ocean_lib):
    """ocean_displace_grid / ocean_grid_tess_levels check their parameters
    first: odd or out-of-range square counts, non-finite scales and texture
    scales beyond +-1e6 (whose texel step would leave the integer range) are
    rejected without a CUDA call."""
    lib = ocean_lib.load()
    bad = [ocean_lib.grid_params(3), ocean_lib.grid_params(0), ocean_lib.grid_params(32768),
           ocean_lib.grid_params(2, float("nan")), ocean_lib.grid_params(2, 64.0, float("inf")),
           ocean_lib.grid_params(2, 1.0e30), ocean_lib.grid_params(2, -2.0e6)]
    for g in bad:
        assert lib.ocean_displace_grid(None, 32, C.byref(g), None, None) == ocean_lib.OCEAN_ERR_INVALID
        assert lib.ocean_grid_tess_levels(C.byref(g), None, None) == ocean_lib.OCEAN_ERR_INVALID
    # shading: a vertex count beyond one launch's 2^31 blocks of 256 (the
    # device addresses are never touched before the count is checked)
    sp = ocean_lib.ocean_shade_params((C.c_float * 3)(0, 10, 0), (C.c_float * 3)(0, -1, 0), (C.c_float * 3)(0, 0, 1), 16)
    for n in (-1, 0x7fffffff * 256 + 1):
        assert lib.ocean_shade_grid(16, n, C.byref(sp), 16, 16, None) == ocean_lib.OCEAN_ERR_INVALID
    rc = lib.ocean_grid_tess_levels(C.byref(ocean_lib.grid_params(2, 1.0e30)), None, None)
    assert rc == ocean_lib.OCEAN_ERR_INVALID
    assert "texcoord_scale" in lib.ocean_last_error().decode()


def test_tuning_table_round_trip(ocean_lib):
    """ocean_get_tuning / ocean_set_tuning: one entry per supported N, values
    replaced for the process and restored, out-of-range values and sizes
    refused.  Host-only (no device call)."""
    for N in (32, 64, 128, 256, 512, 1024, 2048):
        t = ocean_lib.get_tuning(N)
        assert t["row_overlap"] in (0, 1) and t["row_ctas_per_sm"] >= 0 and t["wave_mib"] >= 1
    old = ocean_lib.set_tuning(512, row_overlap=0, row_ctas_per_sm=1, wave_mib=32, col_fused=0, row_variant=1)
    assert ocean_lib.get_tuning(512) == {"row_overlap": 0, "row_ctas_per_sm": 1, "wave_mib": 32, "col_fused": 0,
                                         "row_variant": 1}
    ocean_lib.set_tuning(512, **old)
    assert ocean_lib.get_tuning(512) == old
    for bad in (dict(row_overlap=2), dict(row_ctas_per_sm=-1), dict(wave_mib=0), dict(col_fused=1), dict(col_fused=3),
                dict(row_variant=6), dict(row_variant=-1)):
        with pytest.raises(ocean_lib.OceanError):
            ocean_lib.set_tuning(512, **bad)
    assert ocean_lib.get_tuning(512) == old
    with pytest.raises(ocean_lib.OceanError):
        ocean_lib.get_tuning(48)
    # the fused column kernel exists for N = 512 and 1024 only: elsewhere the
    # entry reads 0 whatever is set
    old2 = ocean_lib.set_tuning(2048, col_fused=2)
    assert ocean_lib.get_tuning(2048)["col_fused"] == 0
    ocean_lib.set_tuning(2048, **old2)
    # 32 x 32 row lines exist at N = 1024 only
    old4 = ocean_lib.set_tuning(2048, row_variant=3)
    assert ocean_lib.get_tuning(2048)["row_variant"] == 0
    ocean_lib.set_tuning(2048, row_variant=4)
    assert ocean_lib.get_tuning(2048)["row_variant"] == 1
    ocean_lib.set_tuning(2048, row_variant=5)
    assert ocean_lib.get_tuning(2048)["row_variant"] == 0
    ocean_lib.set_tuning(2048, **old4)
    # below N = 512 only the every-warp row pass exists
    old3 = ocean_lib.set_tuning(256, row_variant=0)
    assert ocean_lib.get_tuning(256)["row_variant"] == 1
    ocean_lib.set_tuning(256, **old3)
