"""The Fortran binding (fortran/he4g_c.f90) against the C ABI (include/he4g.h):
the bind(C) derived types must list the C structs' fields in the same order
with the same C types, and every bound function must be declared in the
header with the same number of arguments and the same by-value/by-reference
passing. No Fortran compiler exists on either build machine, so this is what
checks the binding."""
import json
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


# ------------------------------------------------------------------ wrappers
WRAP = open(os.path.join(ROOT, "4hetddft-isotropic_gb300", "fortran", "he4g_wrappers.f90")).read()
MODULES = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_modules.json")))["modules"]
FORTRAN_WORDS = set("""subroutine function end use only implicit none real integer logical character type intent in
out inout call if then else return parameter inquire file opened number flush write stop merge max mod
c_null_char c_null_ptr c_associated d0 value""".split())


def _strip(code):
    code = re.sub(r"'[^']*'|\"[^\"]*\"", " ", code)  # strings
    code = "\n".join(line.split("!")[0] for line in code.splitlines())  # comments
    code = re.sub(r"\.(and|or|not|true|false|eq|ne)\.", " ", code, flags=re.I)
    code = re.sub(r"\b\d+(\.\d*)?([de][-+]?\d+)?\b", " ", code, flags=re.I)  # numbers like 1.065d0, 1.d3
    return re.sub(r"%\s*\w+", " ", code)  # derived-type components


def _he4g_c_names():
    names = set(re.findall(r"\b(?:function|subroutine)[ \t]+(\w+)[ \t]*\(", F90))
    names |= set(re.findall(r"type, bind\(C\) :: (\w+)", F90))
    for m in re.finditer(r"^\s*(?:type\(c_ptr\)|logical|integer(?:\(c_int\))?), save :: (.*)$", F90, re.M):
        names |= {p.split("=")[0].strip() for p in m.group(1).split(",")}
    return {n.lower() for n in names}


def wrapper_units():
    return re.findall(r"^subroutine (\w+)\((.*?)\)\n(.*?)^end subroutine", WRAP, re.S | re.M)


def test_wrappers_use_only_variables_the_reference_modules_declare():
    """Every module variable a wrapper names is declared by that module of
    modules.f90, through `use <module>, only:` lists, so that DFT4He3d.f90
    needs no change: the driver's own locals (DFT4He3d.f90:50-146) are out of
    reach of the wrappers."""
    units = wrapper_units()
    assert len(units) >= 7
    for name, _, body in units:
        for mod, only in re.findall(r"^\s*use\s+(\w+)\s*(?:,\s*only\s*:\s*(.*))?$", body, re.M | re.I):
            mod = mod.lower()
            if mod == "he4g_c":
                continue
            assert mod in MODULES, (name, mod)
            assert only, f"{name}: `use {mod}` without an only-list"
            for v in (x.strip().lower() for x in only.split(",")):
                assert v in MODULES[mod], f"{name}: {v} is not a variable of module {mod}"


def test_wrappers_name_nothing_outside_their_modules():
    """Each identifier in a wrapper is a Fortran keyword or intrinsic, a name
    of the he4g_c binding module, a dummy argument or local declaration, or a
    name from its only-lists."""
    c_names = _he4g_c_names()
    subs = {n.lower() for n, _, _ in wrapper_units()}
    for name, args, body in wrapper_units():
        allowed = set(FORTRAN_WORDS) | c_names | subs
        allowed |= {a.strip().lower() for a in args.split(",") if a.strip()}
        for only in re.findall(r"only\s*:\s*(.*)$", body, re.M | re.I):
            allowed |= {x.strip().lower() for x in only.split(",")}
        allowed |= {m.lower() for m in re.findall(r"^\s*use\s+(\w+)", body, re.M | re.I)}
        for decl in re.findall(r"::\s*(.*)$", body, re.M):
            allowed |= {x.split("(")[0].strip().lower() for x in _strip(decl).split(",")}
        code = "\n".join(line for line in _strip(body).splitlines() if not re.match(r"\s*use\b", line, re.I))
        for ident in set(re.findall(r"\b[A-Za-z_]\w*\b", code)):
            assert ident.lower() in allowed, f"{name}: {ident} is neither declared nor use-associated"
    # the defect this guards against: the driver's absorber locals (DFT4He3d.f90:135-137)
    for local in ("lambdah", "txmean", "tzsurf", "pener", "pcurr"):
        assert not re.search(r"\b%s\b" % local, _strip(WRAP), re.I), local
