"""CPU tests of the C-ABI boundary: the library builds and loads, exports
every function include/mo_ed.h declares, the Python mirror binds each of
them, and the host-only helpers match the oracle.  No device compute."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mo_ed.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mo_ed_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def built(pkg):
    import importlib.util
    spec = importlib.util.spec_from_file_location("moed_build", os.path.join(ROOT, "mo-dmft_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build()


def test_header_declares_entry_points():
    fns = header_functions()
    for name in ["mo_ed_create", "mo_ed_multiply_h", "mo_ed_apply_c", "mo_ed_lanczos_iteration",
                 "mo_ed_solve", "mo_ed_calc_green_ftn", "mo_ed_func", "mo_ed_dfunc", "mo_ed_minimization"]:
        assert name in fns


def test_library_exports_every_symbol(built):
    L = C.CDLL(built)
    missing = [f for f in header_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol(pkg, built):
    from importlib import import_module  # noqa: F401
    bound = {n for n, _, _ in pkg.ed.SIGNATURES}
    assert bound == set(header_functions())
    pkg.lib()  # applies every signature


def test_version_and_icom(pkg, built):
    assert pkg.lib().mo_ed_version().decode().startswith("mo_ed")
    from math import comb
    for n in range(16):
        for m in range(n + 1):
            assert pkg.icom(n, m) == comb(n, m)


def test_host_helpers_match_oracle(pkg, oracle, built):
    rng = np.random.default_rng(0)
    norb, nbath = 3, 12
    ns = norb + nbath
    ek, vk, ef = rng.standard_normal(ns), rng.standard_normal((norb, nbath)), rng.standard_normal(norb)
    x = pkg.ev_to_x(ek, vk, ef, ns, nbath)
    assert np.array_equal(x, oracle.ev_to_x(ek, vk, ef, ns, nbath))
    a = pkg.x_to_ev(x, ns, nbath, norb)
    b = oracle.x_to_ev(x, ns, nbath, norb)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)
    with pytest.raises(pkg.EDError):
        pkg.x_to_ev(x[:-1], ns, nbath, norb)


def test_no_device_fails_loudly(pkg, built):
    """Without a CUDA device the solver refuses to start (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(pkg.EDError):
        pkg.EDSolver(0)


def test_fortran_bindings_match_header():
    """Every bind(C) interface of the Fortran module names a declared entry
    point and passes the same number of arguments."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    decl = {}
    for name, args in re.findall(r"\b(mo_ed_\w+)\s*\(([^)]*)\)\s*;", txt):
        decl[name] = 0 if args.strip() in ("", "void") else len(args.split(","))
    f90 = open(os.path.join(ROOT, "mo-dmft_gb300", "fortran", "mo_ed_bind.f90")).read()
    f90 = re.sub(r"&\s*\n\s*", "", f90)
    found = re.findall(r"function\s+(mo_ed_\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(mo_ed_\w+)\"\)", f90)
    assert len(found) >= 20
    for fname, args, cname in found:
        assert fname == cname and cname in decl, cname
        n = 0 if not args.strip() else len(args.split(","))
        assert n == decl[cname], (cname, n, decl[cname])


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c++", "c++11")])
def test_header_compiles_standalone(tmp_path, lang, std):
    """include/mo_ed.h is plain C (and C++ through its extern "C" guard): a host
    of either language includes it with nothing else."""
    import shutil
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include "mo_ed.h"\nint main(void) { mo_ed_options o; (void)o; return 0; }\n')
    r = subprocess.run([cc, "-x", lang, f"-std={std}", "-Wall", "-Wextra", "-pedantic", "-Werror",
                        "-I", os.path.join(ROOT, "include"), "-c", str(src), "-o", str(tmp_path / "u.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_options_layout_matches_header(tmp_path, pkg):
    """mo_ed_options has three copies: the C header, the ctypes mirror
    (ed.Options) and the Fortran bind(C) type (mo_ed_bind.f90).  The same
    fields in the same order with the same kinds, and the ctypes offsets and
    size equal the C compiler's."""
    import shutil
    import subprocess
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no host compiler")
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct\s*\{(.*?)\}\s*mo_ed_options;", txt, re.S).group(1)
    cfields = []   # (name, C type, array length)
    for m in re.finditer(r"\b(int|double)\s+(\w+)(?:\[(\d+)\])?\s*;", body):
        cfields.append((m.group(2), m.group(1), int(m.group(3) or 0)))
    names = [f[0] for f in cfields]
    prog = ['#include <stddef.h>', '#include <stdio.h>', '#include "mo_ed.h"', 'int main(void) {',
            '  printf("%zu\\n", sizeof(mo_ed_options));']
    prog += [f'  printf("%zu\\n", offsetof(mo_ed_options, {n}));' for n in names]
    prog += ['  return 0;', '}']
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(prog) + "\n")
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    size, offs = vals[0], vals[1:]
    # ctypes mirror
    O = pkg.Options
    assert [f[0] for f in O._fields_] == names
    assert C.sizeof(O) == size
    for (n, _), off in zip(O._fields_, offs):
        assert getattr(O, n).offset == off, n
    for (n, ct), (_, ctype, arr) in zip(O._fields_, cfields):
        base = ct._type_ if arr else ct
        assert base == (C.c_int if ctype == "int" else C.c_double), n
        if arr:
            assert ct._length_ == arr, n
    # Fortran bind(C) type: same names, kinds and array lengths, in order
    f90 = open(os.path.join(ROOT, "mo-dmft_gb300", "fortran", "mo_ed_bind.f90")).read()
    tbody = re.search(r"type, bind\(C\) :: mo_ed_options(.*?)end type mo_ed_options", f90, re.S | re.I).group(1)
    ffields = [(m.group(3), m.group(1), int(m.group(4) or 0))
               for m in re.finditer(r"(integer|real)\((c_int|c_double)\)\s*::\s*(\w+)(?:\((\d+)\))?", tbody)]
    assert [f[0] for f in ffields] == names
    for (n, kind, arr), (_, ctype, carr) in zip(ffields, cfields):
        assert (kind == "integer") == (ctype == "int") and arr == carr, n
