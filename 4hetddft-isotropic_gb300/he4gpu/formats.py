"""The reference's on-disk formats, so that its input files and restart files
drive this implementation unchanged.

* Namelist input (DFT4He3d.f90:147-168): ``&input ... /`` with Fortran
  literals (``2.d0``, ``.true.``, ``'Xe_He'``). :func:`read_namelist` parses it
  and :func:`run_from_namelist` maps it onto a run configuration with the
  reference's defaults for everything the file leaves out.
* Density / wave-function files, read by readenc (readenc.f90, modes 0, 2, 3)
  and written by printoutc (printoutc.f90): comment lines starting with ``#``
  (skipped as titols.f90 does), then list-directed records
  ``xmax ymax zmax hx hy hz nx ny nz`` [mode 0: ``limp ximp yimp zimp``],
  [modes 2, 3: ``rimp(3)``, ``vimp(3)``], [mode 3: ``ninvar``, ``invar``], then
  ``den`` (real) or ``psi`` (complex, ``(re,im)``) in Fortran order.
  :func:`read_density` accepts what compilers write in list-directed output:
  values split across lines, ``r*value`` repeat counts and ``D`` exponents.
  :func:`write_density` writes printoutc's header and records.
"""
import re

import numpy as np

# -------------------------------------------------------------- namelist


def _fortran_value(tok):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"":
        return t[1:-1] if t[-1] == t[0] else t[1:]
    low = t.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    num = low.replace("d", "e")
    try:
        if re.fullmatch(r"[+-]?\d+", num):
            return int(num)
        return float(num)
    except ValueError:
        return t


def _split_values(text):
    """Comma/blank separated values of one assignment, quotes kept whole."""
    out, cur, q = [], "", None
    for ch in text:
        if q:
            cur += ch
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
            cur += ch
        elif ch in ", \t\n":
            if cur:
                out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur:
        out.append(cur)
    return out


def read_namelist(source, group="input"):
    """{name (lower case): value} of namelist `group` in a file or text."""
    text = source
    if "\n" not in source and "&" not in source:
        with open(source) as f:
            text = f.read()
    m = re.search(r"&%s\b(.*?)(?:^\s*/\s*$|&end)" % re.escape(group), text, re.S | re.I | re.M)
    if not m:
        raise ValueError(f"namelist &{group} not found")
    body = "\n".join(l.split("!")[0] if "'" not in l and '"' not in l else l for l in m.group(1).splitlines())
    out = {}
    for name, rhs in re.findall(r"([A-Za-z_]\w*(?:\(\s*\d+\s*\))?)\s*=\s*(.*?)(?=(?:[A-Za-z_]\w*(?:\(\s*\d+\s*\))?\s*=)|\Z)",
                                body, re.S):
        vals = [_fortran_value(v) for v in _split_values(rhs)]
        vals = [v for v in vals if v is not None]
        out[name.lower().replace(" ", "")] = vals[0] if len(vals) == 1 else vals
    return out


PS_PER_KELVIN_UNIT = 7.63822291  # DFT4He3d.f90:238 (deltat = deltatps / 7.63822291)


def run_from_namelist(nl):
    """The reference run a namelist describes: config keyword arguments for
    he4gpu.default_config, the impurity table arguments, the initial
    impurity state (A, A*K) and the driver's loop parameters."""
    g = lambda k, d=None: nl.get(k, d)
    cfg = dict(nx=int(g("nx")), ny=int(g("ny", g("nx"))), nz=int(g("nz", g("nx"))),
               xmax=float(g("xmax")), ymax=float(g("ymax", g("xmax"))), zmax=float(g("zmax", g("xmax"))))
    over = {}
    for key, name in [("cp4", "cp4"), ("cpp4", "cpp4"), ("h2o2m4", "h2o2m4"), ("alphas", "alphas"), ("l", "l_alpha"),
                      ("eps4", "eps4"), ("sigma4", "sigma4"), ("lambdah", "lambdah"), ("txmean", "txmean"),
                      ("txsurf", "txsurf"), ("tymean", "tymean"), ("tysurf", "tysurf"), ("tzmean", "tzmean"),
                      ("tzsurf", "tzsurf"), ("mimpur", "mimpur"), ("npd", "npd"), ("icon", "icon")]:
        if key in nl:
            over[name] = nl[key]
    if "lsolid" in nl:
        over["lsolid"] = 1 if nl["lsolid"] else 0
    if "core4" in nl:
        over["core"] = 1 if str(nl["core4"]).strip().upper() == "OTC" else 0
    if "lrk" in nl:
        over["lrk"] = 1 if nl["lrk"] else 0
    deltat = float(g("deltat", 0.0))
    dtps = float(g("deltatps", 0.0))
    if deltat == 0.0 and dtps != 0.0:  # DFT4He3d.f90:233-249
        deltat = dtps / PS_PER_KELVIN_UNIT
    if deltat != 0.0:
        over["deltat"] = deltat
    table = dict(selec=str(g("selec", "Xe_He")).strip(), r_cutoff=float(g("r_cutoff", 2.55)),
                 umax=float(g("umax", 2793.9365463)))
    rimp = np.array([float(g("ximp", 0.0)), float(g("yimp", 0.0)), float(g("zimp", 0.0))])
    # velocities are given in A/ps and stored times 7.63822291 (DFT4He3d.f90:302)
    vimp = np.array([float(g("vximp", 0.0)), float(g("vyimp", 0.0)), float(g("vzimp", 0.0))]) * PS_PER_KELVIN_UNIT
    loop = dict(niter=g("niter"), pener=g("pener", 50), pcurr=g("pcurr"), mode=g("mode", 0), n4=g("n4"),
                filedenin=g("filedenin"), filedenout=g("filedenout"), title=g("title"))
    return cfg, over, table, rimp, vimp, loop


# --------------------------------------------------- list-directed data

_TOKEN = re.compile(r"(\d+)\*\s*(\([^()]*\)|[^\s,()]+)|(\([^()]*\))|([^\s,()]+)")


def _values(text, complex_values):
    """All list-directed values of `text` as a float or complex array."""
    t = text.replace("D", "E").replace("d", "e")
    if "*" not in t:
        flat = np.array(t.translate(str.maketrans("(),", "   ")).split(), dtype=np.float64)
        return flat.view(np.complex128) if complex_values else flat
    out = []
    for m in _TOKEN.finditer(t):
        rep, rv, cv, sv = m.groups()
        tok = rv if rep else (cv or sv)
        n = int(rep) if rep else 1
        if tok.startswith("("):
            a, b = tok[1:-1].split(",")
            v = complex(float(a), float(b))
        else:
            v = float(tok)
        out.extend([v] * n)
    return np.array(out, dtype=np.complex128 if complex_values else np.float64)


def read_density(path, mode=2):
    """A readenc file (modes 0, 2, 3). Returns a dict with the grid record
    (xmax, ymax, zmax, hx, hy, hz, nx, ny, nz), mode 0's limp and impurity
    position, modes 2/3's rimp and vimp, mode 3's invar, and either 'psi'
    (complex, shape (nx, ny, nz), Fortran order) or 'den' (real)."""
    with open(path) as f:
        lines = f.read().splitlines()
    i = 0
    while i < len(lines) and lines[i][:1] == "#":  # titols.f90 with cchar = '#'
        i += 1

    def take(n, complex_values=False):
        """n values from the record starting at line i (list-directed read:
        the rest of the record's last line is skipped)."""
        nonlocal i
        vals = []
        while len(vals) < n:
            if i >= len(lines):
                raise ValueError(f"{path}: file ends before {n} values")
            toks = lines[i].replace(",", " ").split()
            i += 1
            for tok in toks:
                if len(vals) >= n:
                    break
                vals.append(tok)
        return vals

    head = take(13 if mode == 0 else 9)
    out = dict(xmax=float(head[0].replace("D", "E")), ymax=float(head[1].replace("D", "E")),
               zmax=float(head[2].replace("D", "E")), hx=float(head[3].replace("D", "E")),
               hy=float(head[4].replace("D", "E")), hz=float(head[5].replace("D", "E")),
               nx=int(head[6]), ny=int(head[7]), nz=int(head[8]))
    n = out["nx"] * out["ny"] * out["nz"]
    if mode == 0:
        out["limp"] = _fortran_value(head[9])
        out["rimp"] = np.array([float(v.replace("D", "E")) for v in head[10:13]])
    elif mode in (2, 3):
        out["rimp"] = np.array([float(v.replace("D", "E")) for v in take(3)])
        out["vimp"] = np.array([float(v.replace("D", "E")) for v in take(3)])
        if mode == 3:
            ninvar = int(take(1)[0])
            rest = "\n".join(lines[i:])
            vals = _values(rest, True)
            out["invar"] = vals[:ninvar]
            out["psi"] = vals[ninvar:ninvar + n].reshape((out["nx"], out["ny"], out["nz"]), order="F")
            return out
    else:
        raise ValueError(f"readenc mode {mode} is not a file format")
    rest = "\n".join(lines[i:])
    if mode == 0 and "(" not in rest:  # readenc tries den first (readenc.f90:96-99)
        out["den"] = _values(rest, False)[:n].reshape((out["nx"], out["ny"], out["nz"]), order="F")
    else:
        out["psi"] = _values(rest, True)[:n].reshape((out["nx"], out["ny"], out["nz"]), order="F")
    return out


def write_density(path, psi, rimp, vimp, xmax, ymax, zmax, iteration=0, dtps=0.0, time=0.0, selec="Xe_He",
                  r_cutoff=2.55, umax=2793.9365463, cm=(0.0, 0.0, 0.0), npart=0.0, energies=None,
                  ang=(0.0, 0.0, 0.0), r2=(0.0, 0.0, 0.0)):
    """A printoutc file (printoutc.f90): its header, then the grid record,
    rimp, vimp and psi as list-directed records that readenc mode 2 reads
    back. Values are written with 17 significant digits (exact in FP64)."""
    e = dict(ekin4=0.0, elj4=0.0, ealphas=0.0, ecor4=0.0, esolid=0.0, ekinx=0.0, eimpu=0.0, etot=0.0)
    if energies:
        e.update(energies)
    psi = np.asarray(psi, dtype=np.complex128)
    nx, ny, nz = psi.shape
    hx, hy, hz = 2 * xmax / nx, 2 * ymax / ny, 2 * zmax / nz
    f3 = lambda v: "".join(f"{x:16.8E}" for x in v)
    with open(path, "w") as f:
        f.write("#  \n")
        f.write(f"#  Density after {iteration:15d} iterations\n")
        f.write(f"#  Actual deltatps....:{dtps:20.10E}\n")
        f.write(f"#  Total evolution time(ps)...:{time:20.12E}\n")
        f.write(f"#  Impurity potential.........:  {selec}\n")
        f.write(f"#  r_cutoff_gs:{r_cutoff:16.8E}\n")
        f.write(f"#  umax_gs....:{umax:16.8E}\n")
        f.write(f"#  xcm,ycm,zcm:{f3(cm)}\n")
        f.write(f"#  NParticles.:{npart:16.8E}\n")
        for label, key in [("Ekin.......", "ekin4"), ("Elj........", "elj4"), ("Ealphas....", "ealphas"),
                           ("Ecorr......", "ecor4"), ("Esolid.....", "esolid"), ("Ekinx......", "ekinx"),
                           ("Eimpu......", "eimpu"), ("Etot.......", "etot")]:
            f.write(f"#  {label}:{e[key]:16.8E}\n")
        f.write(f"#  <Lx,y,z>...:{f3(ang)}\n")
        f.write(f"#  <x2,y2,z2>.:{f3(r2)}\n")
        f.write("#  \n")
        f.write(" ".join(f"{v:.17E}" for v in (xmax, ymax, zmax, hx, hy, hz)) + f" {nx} {ny} {nz}\n")
        f.write(" ".join(f"{v:.17E}" for v in rimp) + "\n")
        f.write(" ".join(f"{v:.17E}" for v in vimp) + "\n")
        flat = psi.reshape(-1, order="F").view(np.float64)
        per_line = 4  # complex values per line
        full = (flat.size // (2 * per_line)) * 2 * per_line
        if full:
            np.savetxt(f, flat[:full].reshape(-1, 2 * per_line), fmt=" ".join(["(%.17E,%.17E)"] * per_line))
        rest = flat[full:]
        if rest.size:
            f.write(" ".join(f"({rest[k]:.17E},{rest[k + 1]:.17E})" for k in range(0, rest.size, 2)) + "\n")
