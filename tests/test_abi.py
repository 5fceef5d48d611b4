"""CPU checks of the drop-in boundary: the C ABI library loads and exports every function that
include/fedg.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HDR = os.path.join(ROOT, "include", "fedg.h")


def declared():
    txt = open(HDR).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fedg_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_interface():
    names = declared()
    for must in ("fedg_cal_tend_ex", "fedg_cal_vi", "fedg_tint_store_var0", "fedg_tint_store_implicit",
                 "fedg_tint_advance", "fedg_tint_implicit_diagfac", "fedg_modalfilter", "fedg_drhot2pres",
                 "fedg_update", "fedg_ctx_create", "fedg_ctx_destroy", "fedg_guess_train_step"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from fedg import lib as fl

    if not os.path.exists(fl.LIB_PATH):
        import __graft_entry__ as ge

        ge.build()
    lib = ctypes.CDLL(fl.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(fl.EXPORTED) == declared()


def test_error_text_without_gpu():
    """Invalid descriptors are rejected with text before any device work."""
    from fedg import lib as fl

    lib = fl.load()
    h = ctypes.c_void_p()
    d = fl.MeshDesc()
    d.porder = 9
    assert lib.fedg_ctx_create(ctypes.byref(d), ctypes.byref(h)) < 0
    assert b"porder" in lib.fedg_last_error()
    d.porder = 3
    d.NeX = d.NeY = d.NeZ = 2
    d.xmax = d.ymax = d.zmax = 1.0
    d.periodic_x = 0
    d.periodic_y = 1
    assert lib.fedg_ctx_create(ctypes.byref(d), ctypes.byref(h)) < 0
    assert b"periodic" in lib.fedg_last_error()


def test_fortran_shims_bind_declared_symbols():
    """Every bind(C, name=...) of the Fortran shims (not compiled in this image) names a function
    that include/fedg.h declares, and the bind(C) mirrors of the option structs list the C fields
    in the C order."""
    names = set(declared())
    fdir = os.path.join(ROOT, "fe-project_gb300", "fortran")
    bound = []
    for fn in sorted(os.listdir(fdir)):
        if fn.endswith(".F90"):
            bound += re.findall(r'bind\(C,\s*name="([A-Za-z0-9_]+)"\)', open(os.path.join(fdir, fn)).read())
    assert bound
    assert sorted(set(bound) - names) == []
    src = open(os.path.join(fdir, "scale_atm_dyn_dgm_nonhydro3d_gb300.F90")).read()
    hdr = open(HDR).read()
    m = re.search(r"typedef struct \{\s*int eqs, prec, max_iter, use_guess;\s*double dt, tol;\s*\} fedg_update_opts;", hdr)
    assert m, "fedg_update_opts layout changed: update the Fortran mirror"
    assert re.search(r"type, bind\(C\) :: fedg_update_opts\s*integer\(c_int\) :: eqs, prec, max_iter, use_guess\s*"
                     r"real\(c_double\) :: dt, tol\s*end type", src)


def test_c_host_compiles_and_links_every_symbol(tmp_path):
    """A plain C99 host (what a cgo / Fortran / ctypes caller sees) compiles against include/fedg.h
    with -pedantic -Werror and links every declared function from libfedg.so; no GPU call is made."""
    import shutil
    import subprocess

    from fedg import lib as fl

    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    if not os.path.exists(fl.LIB_PATH):
        import __graft_entry__ as ge

        ge.build()
    names = declared()
    src = ['#include <stdio.h>', '#include "fedg.h"', "typedef void (*fn)(void);", "int main(void) {",
           "  const fn f[] = {"]
    src += [f"    (fn)&{n}," for n in names]
    src += ["  };", '  printf("%d\\n", (int)(sizeof f / sizeof f[0]));', "  return 0;", "}"]
    c = tmp_path / "host.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "host"
    libdir = os.path.dirname(fl.LIB_PATH)
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-Wno-cast-function-type",
           "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe), "-L", libdir, "-lfedg",
           f"-Wl,-rpath,{libdir}", f"-Wl,-rpath-link,{cuda_lib}", f"-Wl,-rpath,{cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and int(out.stdout.strip()) == len(names), out.stderr
