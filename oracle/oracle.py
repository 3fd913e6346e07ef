"""ctypes binding of the FP64 CPU oracle (oracle/he4_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, to compare the GPU results with and as the CPU
baseline; the GPU library never uses it. `build()` compiles it with
oracle/Makefile into oracle/_build/.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_D = C.POINTER(C.c_double)
_lib = None


def build(force=False):
    srcs = [os.path.join(HERE, f) for f in ("he4_oracle.c", "he4_oracle.h", "Makefile")]
    srcs.append(os.path.join(os.path.dirname(HERE), "include", "he4g.h"))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in srcs):
        r = subprocess.run(["make", "-B" if force else "-s", "-C", HERE], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else None


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(LIB)
    P = C.c_void_p
    sig = {
        "orc_build_tables": (C.c_int, [P, C.c_char_p, C.c_double, C.c_double, _D, _D, _D, _D]),
        "orc_si": (C.c_double, [C.c_double]),
        "orc_v_xe_he": (C.c_double, [C.c_double]),
        "orc_v_ar_he": (C.c_double, [C.c_double]),
        "orc_v_aziz_he": (C.c_double, [C.c_double]),
        "orc_v_lj_ot": (C.c_double, [C.c_double]),
        "orc_v_alkali_he": (C.c_double, [C.c_double, C.c_int]),
        "orc_v_ag_he": (C.c_double, [C.c_double, C.c_int]),
        "orc_v_ba_he": (C.c_double, [C.c_double]),
        "orc_v_au_he": (C.c_double, [C.c_double]),
        "orc_v_koutselos": (C.c_double, [C.c_double, C.c_int]),
        "orc_select_pot": (C.c_double, [C.c_char_p, C.c_double, C.c_double, C.c_double]),
        "orc_bforce": (C.c_double, [C.c_double, C.c_double, C.c_double]),
        "orc_create": (P, [P, _D, _D, _D, _D]),
        "orc_destroy": (None, [P]),
        "orc_set_threads": (None, [C.c_int]),
        "orc_set_state": (C.c_int, [P, _D, _D, _D]),
        "orc_potenimp": (C.c_int, [P, _D]),
        "orc_poten": (C.c_int, [P]),
        "orc_forceimp": (C.c_int, [P, _D, _D]),
        "orc_steprk": (C.c_int, [P, C.c_double]),
        "orc_steppc": (C.c_int, [P, C.c_double, _D, _D]),
        "orc_step": (C.c_int, [P, C.c_int, _D, _D]),
        "orc_energy": (C.c_int, [P, P]),
        "orc_observables": (C.c_int, [P, C.c_double, P]),
        "orc_get_psi": (C.c_int, [P, _D]),
        "orc_get_den": (C.c_int, [P, _D]),
        "orc_get_field": (C.c_int, [P, C.c_int, _D]),
        "orc_get_impurity": (C.c_int, [P, _D, _D, _D]),
        "orc_get_timec": (C.c_double, [P, C.c_int, C.c_int, C.c_int]),
        "orc_timec_array": (None, [P, _D]),
        "orc_set_uext": (C.c_int, [P, _D]),
        "orc_morse_1d": (C.c_double, [C.c_double]),
        "orc_morse_3d": (C.c_double, [C.c_double, C.c_double, C.c_double]),
        "orc_build_uext": (None, [P, C.c_int, C.c_double, _D]),
        "orc_r2c": (None, [P, _D, _D]),
        "orc_c2r": (None, [P, _D, _D]),
        "orc_deriv_real": (None, [P, C.c_int, C.c_int, _D, _D]),
        "orc_deriv_cplx": (None, [P, C.c_int, C.c_int, _D, _D]),
        "orc_stencil_rows": (None, [C.c_int, _D]),
    }
    for k, (res, args) in sig.items():
        f = getattr(lib, k)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def build_uext(cfg, lsurf3d=False, zsurf=-25.0):
    """The oracle's own surface potential on cfg's grid, (nz, ny, nx)."""
    lib = load()
    out = np.empty((cfg.nz, cfg.ny, cfg.nx))
    lib.orc_build_uext(C.addressof(cfg), 1 if lsurf3d else 0, float(zsurf), _dp(out))
    return out


FIELDS = {"pot4": 0, "dencg": 1, "delj4": 2, "uimp": 3, "dxden": 4, "dyden": 5, "dzden": 6, "ualphas": 7,
          "denalf": 8}


def build_tables(cfg, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463, with_kalfs=True):
    lib = load()
    nh = (cfg.nx // 2 + 1) * cfg.ny * cfg.nz
    fv, wc, po = np.empty(nh), np.empty(nh), np.empty(cfg.npot)
    ka = np.empty(nh) if with_kalfs else None
    lib.orc_build_tables(C.addressof(cfg), selec.encode(), r_cutoff, umax, _dp(fv), _dp(wc), _dp(ka), _dp(po))
    return {"fvlj4": fv, "wcgk": wc, "kalfs": ka, "potion": po}


class OracleRun:
    """The FP64 CPU restatement of one run; same methods as he4gpu.Run."""

    def __init__(self, cfg, tables):
        self.lib = load()
        self.cfg = cfg
        self.shape = (cfg.nz, cfg.ny, cfg.nx)
        ka = tables.get("kalfs")
        self.h = self.lib.orc_create(C.addressof(cfg), _dp(tables["fvlj4"]), _dp(tables["wcgk"]), _dp(ka),
                                     _dp(tables["potion"]))

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, psi, rimp, vimp):
        psi = np.ascontiguousarray(psi, dtype=np.complex128)
        r, v = np.ascontiguousarray(rimp, dtype=float), np.ascontiguousarray(vimp, dtype=float)
        rc = self.lib.orc_set_state(self.h, _dp(psi.view(np.float64)), _dp(r), _dp(v))
        if rc:
            raise RuntimeError(f"oracle set_state: {rc}")

    def potenimp(self, rimp):
        r = np.ascontiguousarray(rimp, dtype=float)
        return self.lib.orc_potenimp(self.h, _dp(r))

    def poten(self):
        return self.lib.orc_poten(self.h)

    def forceimp(self, rimp=(0.0, 0.0, 0.0)):
        r = np.ascontiguousarray(rimp, dtype=float)
        F = np.zeros(3)
        self.lib.orc_forceimp(self.h, _dp(r), _dp(F))
        return F

    def steprk(self, deltat):
        rc = self.lib.orc_steprk(self.h, deltat)
        if rc:
            raise RuntimeError(f"oracle steprk: {rc}")

    def steppc(self, deltat):
        e = np.zeros(2)
        rc = self.lib.orc_steppc(self.h, deltat, _dp(e[:1]), _dp(e[1:]))
        if rc:
            raise RuntimeError(f"oracle steppc: {rc}")
        return float(e[0]), float(e[1])

    def step(self, nsteps=1):
        e = np.zeros(2)
        rc = self.lib.orc_step(self.h, nsteps, _dp(e[:1]), _dp(e[1:]))
        if rc:
            raise RuntimeError(f"oracle step: {rc}")
        return float(e[0]), float(e[1])

    def energy(self):
        from he4gpu.abi import Energies
        en = Energies()
        self.lib.orc_energy(self.h, C.addressof(en))
        return en.as_dict()

    def observables(self, npart):
        from he4gpu.abi import Obs
        o = Obs()
        self.lib.orc_observables(self.h, float(npart), C.addressof(o))
        return {"npart": o.npart, "cm": list(o.cm), "ang": list(o.ang), "ang_im": list(o.ang_im),
                "r2": list(o.r2)}

    @property
    def psi(self):
        out = np.empty(self.shape, dtype=np.complex128)
        self.lib.orc_get_psi(self.h, _dp(out.view(np.float64)))
        return out

    @property
    def den(self):
        out = np.empty(self.shape)
        self.lib.orc_get_den(self.h, _dp(out))
        return out

    def field(self, name):
        out = np.empty(self.shape)
        self.lib.orc_get_field(self.h, FIELDS[name], _dp(out))
        return out

    def impurity(self):
        r, v, a = np.zeros(3), np.zeros(3), np.zeros(3)
        self.lib.orc_get_impurity(self.h, _dp(r), _dp(v), _dp(a))
        return r, v, a

    def timec(self, ix, iy, iz):
        return self.lib.orc_get_timec(self.h, ix, iy, iz)

    def timec_array(self):
        """The driver's timec module array, complex128 (nz, ny, nx)."""
        out = np.empty(self.shape, dtype=np.complex128)
        self.lib.orc_timec_array(self.h, _dp(out.view(np.float64)))
        return out

    def set_uext(self, uext):
        if uext is None:
            self.lib.orc_set_uext(self.h, None)
        else:
            u = np.ascontiguousarray(uext, dtype=np.float64)
            self.lib.orc_set_uext(self.h, _dp(u))

    def r2c(self, a):
        a = np.ascontiguousarray(a, dtype=float)
        out = np.empty((self.cfg.nz, self.cfg.ny, self.cfg.nx // 2 + 1), dtype=np.complex128)
        self.lib.orc_r2c(self.h, _dp(a), _dp(out.view(np.float64)))
        return out

    def c2r(self, s):
        s = np.ascontiguousarray(s, dtype=np.complex128)
        out = np.empty(self.shape)
        self.lib.orc_c2r(self.h, _dp(s.view(np.float64)), _dp(out))
        return out

    def deriv(self, id_, axis, f):
        f = np.ascontiguousarray(f)
        out = np.empty_like(f)
        if np.iscomplexobj(f):
            self.lib.orc_deriv_cplx(self.h, id_, axis, _dp(f.view(np.float64)), _dp(out.view(np.float64)))
        else:
            self.lib.orc_deriv_real(self.h, id_, axis, _dp(f), _dp(out))
        return out
