"""The Fortran binding (fortran/he4g_c.f90) against the C ABI (include/he4g.h):
the bind(C) derived types must list the C structs' fields in the same order
with the same C types, and every bound function must be declared in the
header with the same number of arguments and the same by-value/by-reference
passing. No Fortran compiler exists on either build machine, so this is what
checks the binding."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = open(os.path.join(ROOT, "4hetddft-isotropic_gb300", "fortran", "he4g_c.f90")).read()
HDR = open(os.path.join(ROOT, "include", "he4g.h")).read()

F_TYPES = {"integer(c_int32_t)": "int32_t", "integer(c_int)": "int", "real(c_double)": "double"}


def fortran_type(name):
    m = re.search(r"type, bind\(C\) :: %s\n(.*?)\n\s*end type" % name, F90, re.S)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        t, names = line.split("::")
        ct = F_TYPES[t.strip()]
        fields += [(n.strip(), ct) for n in names.split(",")]
    return fields


def c_struct(name):
    m = re.search(r"typedef struct %s \{(.*?)\} " % name, HDR, re.S)
    assert m, name
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        t, rest = decl.split(None, 1)
        fields += [(n.strip(), t) for n in rest.split(",")]
    return fields


def test_config_layout_matches():
    assert fortran_type("he4g_config") == c_struct("he4g_config")


def test_energies_layout_matches():
    f = [(n.lower(), t) for n, t in fortran_type("he4g_energies")]
    c = [(n.lower(), t) for n, t in c_struct("he4g_energies")]
    assert f == c


def c_prototypes():
    protos = {}
    for m in re.finditer(r"\b(?:int|void|long long|const char\*)\s+(he4g_\w+)\((.*?)\);", HDR, re.S):
        args = [a.strip() for a in m.group(2).replace("\n", " ").split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(1)] = args
    return protos


def test_bound_functions_are_declared_with_matching_arguments():
    protos = c_prototypes()
    funcs = re.findall(r"function (\w+)\((.*?)\) bind\(C, name=\"(\w+)\"\)(.*?)end function", F90, re.S)
    assert len(funcs) >= 10
    for fname, fargs, cname, body in funcs:
        assert cname in protos, cname
        fargs = [a.strip() for a in fargs.split(",") if a.strip()]
        cargs = protos[cname]
        assert len(fargs) == len(cargs), cname
        for fa, ca in zip(fargs, cargs):
            decl = re.search(r"^\s*(.*?)::\s*.*\b%s\b" % re.escape(fa), body, re.M)
            assert decl, (cname, fa)
            by_value = "value" in decl.group(1)
            c_pointer = "*" in ca or "[" in ca
            if "type(c_ptr)" in decl.group(1):
                # an opaque handle or a nullable array: a pointer in C either way
                assert c_pointer or by_value, (cname, fa)
            else:
                assert by_value == (not c_pointer), (cname, fa, ca)
