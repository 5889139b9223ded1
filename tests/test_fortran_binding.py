"""The Fortran host's bind(C) declarations agree with the C header (no compiler needed).

No Fortran compiler exists in the build images, so sccm_gb300/fortran/*.f90 cannot be
compiled here; this test reads them as text and checks, against include/pnamp_gpu.h:
  * each bind(C) derived type has the C struct's fields in the same order with matching
    kinds (int -> integer(c_int), double -> real(c_double), pointer -> type(c_ptr));
  * each bind(C, name=...) interface names a function the header declares, with the
    same number of arguments.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "sccm_gb300", "fortran", "pnamp_gpu.f90")
HDR = os.path.join(ROOT, "include", "pnamp_gpu.h")


def _strip_c_comments(s):
    s = re.sub(r"/\*.*?\*/", "", s, flags=re.S)
    return re.sub(r"//[^\n]*", "", s)


def c_structs():
    s = _strip_c_comments(open(HDR).read())
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", s, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"(const\s+)?(int|double|unsigned int)\s*(.*)", decl)
            assert m, decl
            base = m.group(2)
            for v in m.group(3).split(","):
                v = v.strip()
                kind = "ptr" if v.startswith("*") else ("int" if base == "int" else "double")
                fields.append((v.lstrip("*").strip(), kind))
        out[name] = fields
    return out


def c_functions():
    s = _strip_c_comments(open(HDR).read())
    out = {}
    for name, args in re.findall(r"\b(pnamp_\w+)\s*\(([^;{]*?)\)\s*;", s, flags=re.S):
        args = args.strip()
        out[name] = 0 if args in ("", "void") else len(args.split(","))
    return out


def f_types():
    s = open(F90).read()
    out = {}
    for name, body in re.findall(r"type,\s*bind\(C\)\s*::\s*(\w+)(.*?)end type", s, flags=re.S | re.I):
        fields = []
        for ln in body.splitlines():
            ln = ln.split("!")[0].strip()
            if "::" not in ln:
                continue
            decl, names = ln.split("::")
            kind = "ptr" if "c_ptr" in decl else ("int" if "c_int" in decl else "double")
            fields += [(x.strip(), kind) for x in names.split(",") if x.strip()]
        out[name] = fields
    return out


def f_interfaces():
    s = open(F90).read()
    out = {}
    for m in re.finditer(r"(function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", s, flags=re.I):
        args = [a.strip() for a in m.group(3).split(",") if a.strip()]
        out[m.group(4)] = len(args)
    return out


def test_bind_c_types_match_header_structs():
    cs, ft = c_structs(), f_types()
    for name in ("pnamp_space", "pnamp_hamiltonian", "pnamp_mesh", "pnamp_kernels"):
        assert name in ft, name
        got = [(n.lower(), k) for n, k in ft[name]]
        want = [(n.lower(), k) for n, k in cs[name]]
        assert got == want, f"{name}: Fortran {got} vs C {want}"


def test_bind_c_interfaces_name_header_functions():
    cf, fi = c_functions(), f_interfaces()
    assert len(fi) >= 9
    for name, nargs in fi.items():
        assert name in cf, name
        assert cf[name] == nargs, f"{name}: {nargs} Fortran arguments, {cf[name]} in the header"


def test_shim_keeps_the_reference_signature():
    s = open(os.path.join(ROOT, "sccm_gb300", "fortran", "kernel4triaxial_gpu.f90")).read()
    assert re.search(r"^subroutine Kernel4Triaxial\(lpr, Nphi1, Nphi2, NLEV\)", s, flags=re.M)
    for call in ("pnamp_init", "pnamp_pair", "pnamp_project"):
        assert call + "(" in s
