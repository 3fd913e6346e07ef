"""Generates the golden fixtures that pin the oracle to the reference's own data.

Run where the reference source tree is present, giving its path; the
fixtures it writes are committed, so the tests never need the reference.

* stencil_rows.json: the 13-point first- and second-derivative matrices the
  reference builds at start-up. It reads the Bickley coefficient table
  (blockds.f, COMMON /SDERA/ A(25792)), extracts the M = 13 blocks the way
  newder.f:99-128 does for ICON = 1, and applies the ICON = 13 boundary rewrite
  of redef.f:133-170 (ICON 13 then 12). Coefficients are kept as the decimal
  strings of the table and as the doubles they parse to.
* reference_kats.json: known answers quoted in the reference source
  (V_impur.f90 comments for V_Xe_He(2.0) and V_Ar_He(2.0), the shipped input's
  umax = V_Xe_He(2.55), modules.f90's b4 against bforce), each with file:line.
* reference_modules.json: the variables each module of modules.f90 declares,
  which the Fortran wrappers may use (tests/test_fortran_binding.py).

Usage: python tests/golden/make_golden.py <reference_dir>
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_blockds(path):
    """Returns the 1-based coefficient table A as a dict {index: decimal str}."""
    text = open(path).read().splitlines()
    table = {}
    cur = None
    vals = []
    hdr = re.compile(r"DATA \(A\(I\),I=\s*(\d+),\s*(\d+)\)/")
    num = re.compile(r"[-+]?\d+\.\d+D[-+]\d+")
    for line in text:
        m = hdr.search(line)
        if m:
            cur = (int(m.group(1)), int(m.group(2)))
            vals = []
            continue
        if cur is None:
            continue
        if line.startswith("C"):
            continue
        vals += num.findall(line)
        if len(vals) >= cur[1] - cur[0] + 1:
            for k, v in enumerate(vals[: cur[1] - cur[0] + 1]):
                table[cur[0] + k] = v
            cur = None
    return table


def newder_matrix(A, K, M=13):
    """newder.f:99-128 with ICON = 1: the M x M coefficient matrix (1-based DKF)."""
    ji = 1
    for i in range(3, M - 1, 2):
        ji += (i * i + 1) * (i - 2) // 2 + i
    m2 = M * M
    m21o2 = (m2 + 1) // 2
    ji += m21o2 * (K - 1)
    assert K < M - 1
    sig = 1 - 2 * (K % 2)
    dkf = [None] * (m2 + 2)
    L = ji - 1
    for j in range(1, m21o2):
        L += 1
        dkf[j] = (A[L], 1)
        dkf[m2 - j + 1] = (A[L], sig)
    L += 1
    dkf[m21o2] = (A[L], 1)
    mat = [[dkf[j + (i - 1) * M] for j in range(1, M + 1)] for i in range(1, M + 1)]
    return mat


def redef13(mat):
    """redef.f:151-170 (ICON 13) followed by :133-150 (ICON 12)."""
    k = len(mat)
    ko2 = k // 2
    zero = ("0.0D+00", 1)
    m = [row[:] for row in mat]
    for i in range(ko2, 0, -1):  # rows ko2..1, from row i+1 shifted left
        src = m[i]  # row i+1 (0-based index i)
        m[i - 1] = [src[j + 1] for j in range(k - 1)] + [zero]
    for i in range(ko2 + 2, k + 1):  # rows ko2+2..k, from row i-1 shifted right
        src = m[i - 2]
        m[i - 1] = [zero] + [src[j - 1] for j in range(1, k)]
    return m


def module_variables(path):
    """{module: sorted variable names} of modules.f90: the names each module
    declares at module level (entity lists of its declaration statements,
    initialisers and array specs removed; components of derived types
    excluded)."""
    mods, cur, in_type = {}, None, False
    for line in open(path, encoding="latin-1").read().splitlines():
        code = line.split("!")[0]
        if re.match(r"\s*module\s+\w+\s*$", code, re.I):
            cur = code.split()[1].lower()
            mods[cur] = set()
            continue
        if re.match(r"\s*end\s*module", code, re.I):
            cur = None
            continue
        if cur is None:
            continue
        if re.match(r"\s*type\s*(,|::|\s+\w+\s*$)", code, re.I) and "(" not in code.split("::")[0][4:]:
            in_type = True
            continue
        if re.match(r"\s*end\s*type", code, re.I):
            in_type = False
            continue
        if in_type or "::" not in code:
            continue
        rhs = code.split("::", 1)[1]
        while re.search(r"\([^()]*\)", rhs):
            rhs = re.sub(r"\([^()]*\)", "", rhs)
        rhs = re.sub(r"'[^']*'|\"[^\"]*\"", "", rhs)
        for part in rhs.split(","):
            name = part.split("=")[0].strip()
            if re.match(r"^[A-Za-z_]\w*$", name):
                mods[cur].add(name.lower())
    return {k: sorted(v) for k, v in mods.items()}


def signed_decimal(entry):
    s, sg = entry
    if sg > 0:
        return s
    return s[1:] if s.startswith("-") else "-" + s.lstrip("+")


def to_float(entry):
    s, sg = entry
    v = float(s.replace("D", "E"))
    return sg * v


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference source tree>")
    ref = sys.argv[1]
    A = parse_blockds(os.path.join(ref, "blockds.f"))
    out = {"source": "blockds.f via newder.f:99-128 (ICON=1) and redef.f:133-170 (ICON=13)"}
    for K, name in ((1, "d1"), (2, "d2")):
        raw = newder_matrix(A, K)
        mat = redef13(raw)
        out[name] = {
            "centre_row_decimal": [signed_decimal(e) for e in raw[6]],
            "centre_row": [to_float(e) for e in raw[6]],
            "matrix_icon13": [[to_float(e) for e in row] for row in mat],
        }
    with open(os.path.join(HERE, "stencil_rows.json"), "w") as f:
        json.dump(out, f, indent=1)

    # known answers quoted in the reference source
    def grep(fname, pat):
        lines = open(os.path.join(ref, fname), encoding="latin-1").read().splitlines()
        for i, line in enumerate(lines, 1):
            m = re.search(pat, line)
            if m:
                return i, m.group(1)
        raise RuntimeError(f"{pat} not found in {fname}")

    kats = []
    ln, v = grep("V_impur.f90", r"r_cutoff = 2\.0d0; umax = (21450\.\d+)d0")
    kats.append({"what": "V_Xe_He(2.0)", "value": float(v), "rel_tol": 1e-12, "source": f"V_impur.f90:{ln}"})
    ln, v = grep("V_impur.f90", r"r_cutoff = 2\.0d0; umax = (8\.0808095081)d3")
    kats.append({"what": "V_Ar_He(2.0)", "value": float(v) * 1e3, "rel_tol": 1e-10,
                 "source": f"V_impur.f90:{ln}"})
    ln, v = grep("input_files/xe-he1000-hoc-200mps.input", r"umax = (2\.7939365463E\+03)")
    kats.append({"what": "V_Xe_He(2.55)", "value": float(v), "rel_tol": 1e-10,
                 "source": f"input_files/xe-he1000-hoc-200mps.input:{ln}"})
    ln, v = grep("modules.f90", r"b4 =(-?\d+\.\d+)d0")
    kats.append({"what": "bforce_OT(eps4=10.22, sigma4=2.556, h4ot=2.190323)", "value": float(v),
                 "abs_tol": 0.005, "source": f"modules.f90:{ln}"})
    with open(os.path.join(HERE, "reference_kats.json"), "w") as f:
        json.dump(kats, f, indent=1)
    with open(os.path.join(HERE, "reference_modules.json"), "w") as f:
        json.dump({"source": "modules.f90", "modules": module_variables(os.path.join(ref, "modules.f90"))}, f,
                  indent=1)
    print("wrote stencil_rows.json, reference_kats.json and reference_modules.json")


if __name__ == "__main__":
    main()
