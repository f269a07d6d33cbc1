"""The C ABI without a GPU: the library builds for sm_103a, loads, and exports
every entry point include/npbmz.h and include/npbmz_lu.h declare; a C99
consumer compiles and links against both headers; the Julia ccalls and the
Python ctypes declarations match the prototypes; the package never reaches
the oracle and creates no handle without a device; and the host-side helpers
(zone set-up, seeded coefficients, layouts) agree with the oracle."""
import json
import re
from pathlib import Path

import numpy as np
import pytest

import npbmz

INCLUDE = Path(__file__).resolve().parents[1] / "include"
HEADER = INCLUDE / "npbmz.h"
LU_HEADER = INCLUDE / "npbmz_lu.h"


def declared_functions(header=HEADER):
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(npbmz_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_exported_list():
    from npbmz import lu

    assert sorted(npbmz.EXPORTS) == declared_functions()
    assert sorted(lu.LU_EXPORTS) == declared_functions(LU_HEADER)


def test_every_header_is_covered():
    assert sorted(p.name for p in INCLUDE.glob("*.h")) == ["npbmz.h", "npbmz_lu.h"]


def test_library_exports_every_declared_symbol(npbmz_mod):
    L = npbmz_mod.lib()
    for header in (HEADER, LU_HEADER):
        for name in declared_functions(header):
            assert hasattr(L, name), name


def test_headers_compile_and_link_as_c(npbmz_mod, tmp_path):
    """A C99 consumer (what a ccall, cgo or ctypes binding sees) compiles
    against both headers with every warning an error, takes the address of
    every declared entry point, links against libnpbmz_gpu.so, and runs the
    calls that need no device: zone set-up and the NULL-handle errors."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = declared_functions(HEADER) + declared_functions(LU_HEADER)
    src = tmp_path / "consumer.c"
    src.write_text(
        "#include <stdio.h>\n#include <string.h>\n"
        '#include "npbmz.h"\n#include "npbmz_lu.h"\n'
        "typedef void (*fn)(void);\n"
        "static const fn entry[] = {" + ", ".join(f"(fn){n}" for n in names) + "};\n"
        "int main(void) {\n"
        "  int nx[16], ny[16], nz[16], nbr[64], i;\n"
        "  for (i = 0; i < (int)(sizeof entry / sizeof entry[0]); ++i) if (!entry[i]) return 10;\n"
        "  if (npbmz_zone_setup(NPBMZ_BT, 24, 24, 6, 2, 2, 1.0, nx, ny, nz, nbr) != 0) return 11;\n"
        "  if (nx[0] != 12 || ny[3] != 12 || nz[2] != 6) return 12;\n"
        "  if (npbmz_lu_zone_setup(24, 24, 6, 4, 4, 1.0, nx, ny, nz, nbr) != 0) return 13;\n"
        "  if (nx[15] != 6 || nbr[0] != 12) return 14;\n"
        "  if (npbmz_lu_ssor(NULL, 0) >= 0) return 15;\n"
        '  if (strcmp(npbmz_lu_last_error(NULL), "null handle") != 0) return 16;\n'
        "  if (npbmz_lu_zone_setup(25, 24, 6, 4, 4, 1.0, nx, ny, nz, nbr) == 0) return 17;\n"
        '  if (!strstr(npbmz_lu_last_error(NULL), "equal zones")) return 18;\n'
        '  printf("c consumer ok\\n");\n'
        "  return 0;\n}\n")
    libdir = npbmz_mod.lib_path().parent
    exe = tmp_path / "consumer"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{INCLUDE}", str(src), "-o", str(exe),
                    f"-L{libdir}", "-lnpbmz_gpu", f"-Wl,-rpath,{libdir}"], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "c consumer ok" in r.stdout, (r.returncode, r.stdout, r.stderr)


def test_no_device_means_no_handle(npbmz_mod):
    """Without a CUDA device the library refuses to create a problem, with the
    CUDA error in its text: there is no CPU fallback to run instead."""
    from npbmz import lu

    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(npbmz.NpbmzError, match="CUDA|cuda"):
        lu.LuProblem.from_class("S")
    with pytest.raises(npbmz.NpbmzError, match="CUDA|cuda"):
        npbmz.Problem.from_class("BT", "S")


def test_library_is_built_for_sm_103a():
    from npbmz import build

    assert "arch=compute_103a,code=sm_103a" in build.ARCH


@pytest.mark.parametrize("kind,cls", [("BT", c) for c in "SWABC"] + [("SP", c) for c in "SWABC"])
def test_zone_setup_matches_oracle(npbmz_mod, oracle_mod, kind, cls):
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    k = npbmz.KINDS[kind]
    a = npbmz.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    b = oracle_mod.zone_setup(k, gx, gy, gz, xz, yz, ratio)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    nx, ny, nz, nbr = a
    assert int(np.sum(nx[:xz])) == gx and int(np.sum(ny[::xz])) == gy


def test_bt_class_b_zone_widths():
    """The geometric widths of BT class B (the 304x208x17 grid in 8x8 zones)."""
    nx, ny, nz, nbr = npbmz.zone_setup(npbmz.BT, 304, 208, 17, 8, 8, 4.5)
    assert nx[:8].tolist() == [16, 20, 24, 30, 38, 47, 57, 72]
    assert ny[::8].tolist() == [11, 13, 17, 21, 26, 31, 40, 49]
    area = nx * ny
    assert 20.0 < area.max() / area.min() < 20.1


def test_periodic_neighbours():
    nx, ny, nz, nbr = npbmz.zone_setup(npbmz.BT, 24, 24, 6, 2, 2, 3.0)
    # zone 0 = (i=1,j=1): west/east are zone 1, south/north are zone 2
    assert nbr[:4].tolist() == [1, 1, 2, 2]
    nx2, ny2, nz2, nbr2 = npbmz.zones_from_widths([8, 16], [10, 14], 6)
    assert nbr2.tolist() == nbr.tolist()
    assert nx2.tolist() == [8, 16, 8, 16] and ny2.tolist() == [10, 10, 14, 14]


@pytest.mark.parametrize("seed", [0, 1, 7, 12345])
def test_seeded_coefficients_positivity_rule(npbmz_mod, seed):
    nx, ny, nz, nbr = npbmz.zone_setup(npbmz.BT, 304, 208, 17, 8, 8, 4.5)
    ce, e = npbmz.seeded_coefficients(seed, nx, ny, nz, 304, 208, 17, 8, 8)
    assert e >= 0
    assert np.all(ce[:4] >= 0.5) and np.all(ce[:4] < 2.0)
    assert np.all(ce[4] >= 0.5 * 2 ** e) and np.all(ce[4] < 2.0 * 2 ** e)
    ce2, e2 = npbmz.seeded_coefficients(seed, nx, ny, nz, 304, 208, 17, 8, 8)
    np.testing.assert_array_equal(ce, ce2)


@pytest.mark.parametrize("kind,cls,seed", [("BT", "C", 20261203), ("SP", "C", 20261203), ("BT", "B", 3),
                                           ("SP", "A", 3), ("BT", "S", 0), ("BT", "W", 99)])
def test_seeded_coefficients_match_the_oracle(npbmz_mod, oracle_mod, kind, cls, seed):
    """The library's seeded coefficients (host code of libnpbmz_gpu.so) and
    the oracle's own restatement (which the bench's reference arm uses, so
    that arm loads no product library) give the same ce and energy scale."""
    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES[kind][cls]
    nx, ny, nz, nbr = oracle_mod.zone_setup(npbmz.KINDS[kind], gx, gy, gz, xz, yz, ratio)
    a, ea = npbmz.seeded_coefficients(seed, nx, ny, nz, gx, gy, gz, xz, yz)
    b, eb = oracle_mod.seeded_coefficients(seed, nx, ny, nz, gx, gy, gz, xz, yz)
    assert ea == eb
    np.testing.assert_array_equal(a, b)
    if (cls, seed) == ("C", 20261203):
        assert ea == 2  # the benchmark's energy-row scale 2^2


@pytest.mark.parametrize("params,text", [
    ([float("nan"), 24, 24, 6, 2, 2], b"dt"), ([float("inf"), 24, 24, 6, 2, 2], b"dt"),
    ([0.01, 1, 24, 6, 2, 2], b"at least 2"), ([0.01, 24, 24, 1, 2, 2], b"at least 2"),
    ([0.01, 24, 24, 6, 0, 2], b"zone"), ([0.01, 24, 24, 6, 2, 2.5], b"whole")])
def test_noalloc_rejects_bad_parameters_before_any_cuda_call(npbmz_mod, params, text):
    """npbmz_bt_xsolve_noalloc checks dt and the grid constants as
    npbmz_create does, before it touches the GPU (so this runs without one)."""
    import ctypes

    L = npbmz.lib()
    a = np.array(params, np.float64)
    buf = np.zeros(8)
    rc = L.npbmz_bt_xsolve_noalloc(8, 10, 6, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   ctypes.c_void_p(buf.ctypes.data), ctypes.c_void_p(buf.ctypes.data), None)
    assert rc == -1
    assert text in L.npbmz_last_error(None)


def test_ref_layout_sizes():
    # BT u carries the 2-deep halo on i, j, k; SP pads i, j to odd extents
    assert npbmz.ref_elems(npbmz.BT, npbmz.U, 8, 10, 6) == 5 * 13 * 15 * 11
    assert npbmz.ref_elems(npbmz.BT, npbmz.RHS, 8, 10, 6) == 5 * 10 * 12 * 8
    assert npbmz.ref_elems(npbmz.BT, npbmz.FORCING, 8, 10, 6) == 5 * 9 * 11 * 7
    assert npbmz.ref_elems(npbmz.SP, npbmz.U, 12, 12, 6) == 5 * 17 * 17 * 11
    assert npbmz.ref_elems(npbmz.SP, npbmz.RHS, 12, 12, 6) == 5 * 13 * 13 * 7


@pytest.mark.parametrize("cls", list("SWABCD"))
def test_lu_zone_setup_matches_oracle(npbmz_mod, oracle_mod, cls):
    from npbmz import lu

    niter, dt, ratio, xz, yz, gx, gy, gz = npbmz.CLASSES["LU"][cls]
    a = lu.lu_zone_setup(gx, gy, gz, xz, yz, ratio)
    b = oracle_mod.lu_zone_setup(gx, gy, gz, xz, yz, ratio)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_lu_zone_setup_rejects_non_integer_extents(npbmz_mod):
    from npbmz import lu

    with pytest.raises(npbmz.NpbmzError, match="do not split into 4 equal zones"):
        lu.lu_zone_setup(25, 24, 6, 4, 4)


def test_lu_calls_without_a_handle_report_an_error(npbmz_mod):
    """A NULL handle is an error with text, read from npbmz_lu_last_error(NULL)
    (no device work: the call returns before touching CUDA)."""
    from npbmz import lu

    L = lu.lib()
    assert L.npbmz_lu_ssor(None, 0) < 0
    assert L.npbmz_lu_last_error(None) == b"null handle"
    with pytest.raises(npbmz.NpbmzError, match="outside the zones"):
        lu.lu_zone_setup(24, 24, 6, 3, 2)


def test_julia_bindings_call_only_declared_entry_points():
    """The Julia binding and shim (written against the ABI; Julia is not
    installed here) name only functions the headers declare, and the LU
    binding covers the LU time loop's calls."""
    jl = Path(__file__).resolve().parents[1] / "npbapps.jl_gb300" / "julia"
    declared = set(declared_functions(HEADER)) | set(declared_functions(LU_HEADER))
    called = set()
    for f in jl.glob("*.jl"):
        called |= set(re.findall(r"ccall\(\(:(npbmz_[a-z_0-9]+)\s*,", f.read_text()))
    assert called and called <= declared, sorted(called - declared)
    for name in ("npbmz_lu_create", "npbmz_lu_setup", "npbmz_lu_exch_qbc", "npbmz_lu_ssor", "npbmz_lu_iterate",
                 "npbmz_lu_verify", "npbmz_lu_upload", "npbmz_lu_download", "npbmz_lu_destroy"):
        assert name in called, name


SHIM_METHODS = {"NPBApps.BT.adi": "BT.adi", "NPBApps.SP.adi": "SP.adi", "$M.exch_qbc": ("BT.exch_qbc", "SP.exch_qbc"),
                "NPBApps.LU.ssor": "LU.ssor", "NPBApps.LU.exch_qbc": "LU.exch_qbc"}


def shim_parameters(text, name):
    """(name, type) of each positional parameter of the shim method `name`,
    with a trailing Vararg{Any,N} expanded into N untyped entries."""
    m = re.search(re.escape(name) + r"\((.*?)\)\n", text, re.S)
    assert m, name
    out = []
    for a in (x.strip() for x in re.split(r",(?![^{]*\})", m.group(1))):
        if not a:
            continue
        v = re.fullmatch(r"\w+::Vararg\{Any,\s*(\d+)\}", a)
        if v:
            out += [("", None)] * int(v.group(1))
            continue
        nm, _, ty = a.partition("::")
        out.append((nm.strip(), ty.strip() or None))
    return out


def test_julia_shim_dispatches_at_the_reference_argument_positions():
    """Every DeviceZone / LuDeviceZone-typed parameter of the shim sits at the
    position where the reference function takes the array of that name, and
    each method has the reference's arity.  The reference parameter lists come
    from the committed fixture tests/golden/reference_signatures.json, which
    tests/golden/make_reference_signatures.py extracts from the function
    headers (src/BT/adi.jl:5, src/SP/adi.jl:6, src/BT/exchange_qbc.jl:1,
    src/SP/exchange_qbc.jl:1, src/LU/ssor.jl:9, src/LU/exchange_qbc.jl:17)."""
    root = Path(__file__).resolve().parents[1]
    text = (root / "npbapps.jl_gb300" / "julia" / "NPBAppsGPUShim.jl").read_text()
    ref = json.loads((root / "tests" / "golden" / "reference_signatures.json").read_text())
    for name, keys in SHIM_METHODS.items():
        params = shim_parameters(text, name)
        typed = [(i, nm, ty) for i, (nm, ty) in enumerate(params) if ty and "DeviceZone" in ty]
        assert typed, name
        for key in (keys if isinstance(keys, tuple) else (keys,)):
            want = ref[key]["params"]
            assert len(params) == len(want), (name, len(params), key, len(want))
            for i, nm, ty in typed:
                assert want[i] == nm, f"{name}: {nm}::{ty} at position {i + 1}; {ref[key]['file']} has {want[i]}"


def _zone_geometries(seed, count, square=False):
    """Seeded random splits: equal zones (extent a multiple of the zone count)
    and geometric ones (ratio in [1.5, 6]); square: x_zones == y_zones."""
    rng = np.random.default_rng(seed)
    for _ in range(count):
        xz, yz = (int(v) for v in rng.integers(2, 17, size=2))
        if square:
            yz = xz
        if rng.random() < 0.5:
            gx, gy, ratio = xz * int(rng.integers(3, 40)), yz * int(rng.integers(3, 40)), 1.0
        else:
            gx, gy = (int(v) for v in rng.integers(16 * max(xz, yz), 40 * max(xz, yz) + 1, size=2))
            ratio = float(rng.uniform(1.5, 6.0))
        yield gx, gy, int(rng.integers(3, 40)), xz, yz, ratio


def test_zone_setup_properties_on_random_splits(npbmz_mod, oracle_mod):
    """300 seeded splits, BT/SP rule: the library's zone_setup equals the
    oracle's, the widths tile the grid, and the neighbour table is the
    periodic one (the east neighbour's west neighbour is the zone itself)."""
    for gx, gy, gz, xz, yz, ratio in _zone_geometries(11, 300):
        a = npbmz.zone_setup(npbmz.BT, gx, gy, gz, xz, yz, ratio)
        b = oracle_mod.zone_setup(oracle_mod.KIND_BT, gx, gy, gz, xz, yz, ratio)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y, err_msg=str((gx, gy, gz, xz, yz, ratio)))
        nx, ny, nz, nbr = a
        w = nbr.reshape(-1, 4)
        assert nx.reshape(yz, xz)[0].sum() == gx and ny.reshape(yz, xz)[:, 0].sum() == gy
        assert np.all(nz == gz)
        z = np.arange(xz * yz)
        assert np.array_equal(w[w[z, 1], 0], z) and np.array_equal(w[w[z, 3], 2], z)
        assert np.array_equal(w[z, 1], (z // xz) * xz + (z % xz + 1) % xz)


def test_lu_zone_setup_properties_on_random_splits(oracle_mod):
    """200 seeded square splits (LU's neighbour rule assumes x_zones ==
    y_zones), LU rule: the library equals the oracle, the widths tile the grid,
    and south/north and west/east are inverse pairs."""
    from npbmz import lu

    for gx, gy, gz, xz, _, ratio in _zone_geometries(12, 200, square=True):
        a = lu.lu_zone_setup(gx, gy, gz, xz, xz, ratio)
        b = oracle_mod.lu_zone_setup(gx, gy, gz, xz, xz, ratio)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y, err_msg=str((gx, gy, gz, xz, ratio)))
        nx, ny, nz, nbr = a
        w = nbr.reshape(-1, 4)
        assert nx.reshape(xz, xz)[0].sum() == gx and ny.reshape(xz, xz)[:, 0].sum() == gy
        z = np.arange(xz * xz)
        assert np.array_equal(w[w[z, 1], 0], z) and np.array_equal(w[w[z, 3], 2], z)


def _c_prototypes():
    """{name: (return type, [parameter types])} of both headers."""
    protos = {}
    for header in (HEADER, LU_HEADER):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
        for ret, name, params in re.findall(r"([A-Za-z_][\w \t*]*?)\s*\b(npbmz_\w+)\s*\(([^)]*)\)\s*;", text):
            types = []
            for prm in params.split(","):
                prm = " ".join(prm.split())
                if prm and prm != "void":
                    types.append(re.sub(r"\b\w+$", "", prm).replace(" *", "*").strip())
            protos[name] = (ret.strip(), types)
    return protos


def _julia_ccalls(text):
    """(name, return type, [argument types]) of every ccall into libnpbmz."""
    def split_top(s):
        out, depth, cur = [], 0, ""
        for ch in s:
            if ch in "({":
                depth += 1
            elif ch in ")}":
                depth -= 1
            if ch == "," and depth == 0:
                out.append(cur.strip())
                cur = ""
            else:
                cur += ch
        if cur.strip():
            out.append(cur.strip())
        return out

    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+),\s*libnpbmz\),\s*", text):
        rest = text[m.end():]
        ret = rest[:rest.index(",")].strip()
        rest = rest[rest.index(",") + 1:].lstrip()
        assert rest.startswith("("), m.group(1)
        depth = 0
        for i, ch in enumerate(rest):
            depth += ch == "("
            depth -= ch == ")"
            if depth == 0:
                break
        calls.append((m.group(1), ret, split_top(rest[1:i])))
    return calls


_JULIA_SCALAR = {"Cint": "int", "Cdouble": "double", "UInt64": "uint64_t", "Csize_t": "size_t"}


def _compatible(c_type, jl_type):
    if "*" in c_type:
        base = c_type.replace("const ", "").rstrip("*").strip()
        if c_type.count("*") == 2:
            return jl_type in ("Ptr{Ptr{Cvoid}}", "Ref{Ptr{Cvoid}}")
        if jl_type == "Ptr{Cvoid}":
            return True
        want = {"double": ("Ptr{Cdouble}", "Ref{Cdouble}"), "int": ("Ptr{Cint}", "Ref{Cint}"),
                "int64_t": ("Ptr{Int64}", "Ref{Int64}"), "char": ("Cstring", "Ptr{UInt8}")}.get(base, ())
        return jl_type in want
    return _JULIA_SCALAR.get(jl_type) == c_type


def test_julia_ccalls_match_the_c_prototypes():
    """Every ccall in the Julia binding passes as many arguments as the C
    prototype declares, each of a compatible type, and expects its return
    type (Julia is not installed here, so this is the check its calls get)."""
    protos = _c_prototypes()
    julia = Path(__file__).resolve().parents[1] / "npbapps.jl_gb300" / "julia"
    n = 0
    for f in sorted(julia.glob("*.jl")):
        for name, ret, args in _julia_ccalls(f.read_text()):
            c_ret, c_args = protos[name]
            assert len(args) == len(c_args), (f.name, name, args, c_args)
            for c, j in zip(c_args, args):
                assert _compatible(c, j), (f.name, name, c, j)
            assert (ret == "Cint") if c_ret == "int" else (ret in ("Cstring", "Ptr{UInt8}")), (f.name, name, ret)
            n += 1
    assert n >= 30


def _ctypes_compatible(c_type, ct):
    import ctypes

    if "*" in c_type:
        base = c_type.replace("const ", "").rstrip("*").strip()
        if c_type.count("*") == 2:
            return ct is ctypes.POINTER(ctypes.c_void_p)
        if ct is ctypes.c_void_p:
            return True
        want = {"double": ctypes.POINTER(ctypes.c_double), "int": ctypes.POINTER(ctypes.c_int),
                "int64_t": ctypes.POINTER(ctypes.c_int64), "char": ctypes.c_char_p}.get(base)
        return ct is want
    return ct is {"int": ctypes.c_int, "double": ctypes.c_double, "uint64_t": ctypes.c_uint64,
                  "size_t": ctypes.c_size_t, "int64_t": ctypes.c_int64}[c_type]


def test_python_ctypes_declarations_match_the_c_prototypes(npbmz_mod):
    """The ctypes binding declares every entry point of both headers with the
    prototype's argument count, compatible argument types and return type."""
    from npbmz import lu

    L = npbmz_mod.lib()
    lu.lib()
    for name, (c_ret, c_args) in _c_prototypes().items():
        f = getattr(L, name)
        assert f.argtypes is not None, name
        assert len(f.argtypes) == len(c_args), (name, f.argtypes, c_args)
        for c, ct in zip(c_args, f.argtypes):
            assert _ctypes_compatible(c, ct), (name, c, ct)
        assert _ctypes_compatible(c_ret, f.restype), (name, c_ret, f.restype)


def test_the_product_never_reaches_the_oracle(npbmz_mod):
    """The oracle is test infrastructure: no module of the package imports it,
    no CUDA/C++ source includes it, the build does not link it, and the built
    library depends on the CUDA runtime and the C/C++ runtimes only."""
    import ast
    import subprocess

    pkg = Path(__file__).resolve().parents[1] / "npbapps.jl_gb300"
    for f in pkg.rglob("*.py"):
        for node in ast.walk(ast.parse(f.read_text())):
            if isinstance(node, ast.Import):
                mods = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                mods = [node.module or ""]
            else:
                continue
            assert not any(m.split(".")[0] == "oracle" for m in mods), (f, mods)
    for f in list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")) + list(pkg.rglob("*.h")):
        for inc in re.findall(r'#\s*include\s*[<"]([^>"]+)[>"]', f.read_text()):
            assert "oracle" not in inc, (f, inc)
    assert "oracle" not in (pkg / "npbmz" / "build.py").read_text()
    out = subprocess.run(["readelf", "-d", str(npbmz_mod.lib_path())], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("readelf unavailable")
    needed = re.findall(r"\(NEEDED\)\s+Shared library: \[([^\]]+)\]", out.stdout)
    assert needed and all(re.match(r"lib(cudart|stdc\+\+|m|gcc_s|c|dl|pthread|rt)\.so|ld-linux", n) for n in needed), needed
