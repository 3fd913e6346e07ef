"""Host-side mirror of the reference's time-step routines over libhe4g.so.

`Run` carries the names and argument meaning of the reference routines it
replaces (steprk.f90, steppc.f90, potenimp.f90, poten.f90, energy.f90,
r_cm.f90, the loop body of DFT4He3d.f90:840-852) and raises `He4gError`
where the reference would STOP. All arithmetic runs in libhe4g.so on the GPU;
this module only moves arguments across the C ABI.
"""
import ctypes as C

import numpy as np

from . import abi
from .abi import CORE_OT, CORE_OTC, Config  # noqa: F401
from .initial import (PS_TO_K, KELVIN_PER_PS, woods_saxon_psi, collision_case,  # noqa: F401
                      config_for_case, make_meta, state_for, batch_cases, serve_stream)


NTILES = 5  # HE4G_NTILES


class He4gError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"he4g error {code} ({abi.ERRORS.get(code, '?')}): {msg}")
        self.code = code


def default_config(nx, ny, nz, xmax, ymax=None, zmax=None, **overrides):
    """Reference defaults (he4g_default_config) with keyword overrides."""
    lib = abi.load()
    cfg = Config()
    ymax = xmax if ymax is None else ymax
    zmax = xmax if zmax is None else zmax
    lib.he4g_default_config(C.byref(cfg), nx, ny, nz, xmax, ymax, zmax)
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


def reference_config(nx, ny, nz, xmax, ymax=None, zmax=None, **overrides):
    """default_config computed in Python (abi.reference_defaults) without
    loading libhe4g.so: for processes that only run the CPU oracle."""
    ymax = xmax if ymax is None else ymax
    zmax = xmax if zmax is None else zmax
    cfg = abi.reference_defaults(nx, ny, nz, xmax, ymax, zmax)
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise KeyError(k)
        setattr(cfg, k, v)
    return cfg


def footprint(cfg):
    """Device bytes a run of this configuration allocates (he4g_footprint)."""
    lib = abi.load()
    b = C.c_uint64()
    rc = lib.he4g_footprint(C.byref(cfg), C.byref(b))
    if rc:
        raise He4gError(rc, "footprint")
    return int(b.value)


def build_tables(cfg, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463, with_kalfs=None):
    """fforma / initcg / kalfs / potenimpini tables of the run (host side)."""
    lib = abi.load()
    nh = (cfg.nx // 2 + 1) * cfg.ny * cfg.nz
    fv = np.empty(nh)
    wc = np.empty(nh)
    if with_kalfs is None:
        with_kalfs = cfg.core == CORE_OTC
    ka = np.empty(nh) if with_kalfs else None
    po = np.empty(cfg.npot)
    rc = lib.he4g_build_tables(C.byref(cfg), selec.encode(), r_cutoff, umax, abi.dptr(fv), abi.dptr(wc),
                               abi.dptr(ka) if ka is not None else None, abi.dptr(po))
    if rc:
        raise He4gError(rc, "build_tables")
    return {"fvlj4": fv, "wcgk": wc, "kalfs": ka, "potion": po}


def build_uext(cfg, lsurf3d=False, zsurf=-25.0):
    """The TiO2 surface potential of DFT4He3d.f90:760-784 (morse.f90) on the
    run's grid, shape (nz, ny, nx); zsurf defaults to the driver's -25 A."""
    lib = abi.load()
    out = np.empty((cfg.nz, cfg.ny, cfg.nx))
    rc = lib.he4g_build_uext(C.byref(cfg), 1 if lsurf3d else 0, float(zsurf), abi.dptr(out))
    if rc:
        raise He4gError(rc, "build_uext")
    return out


def build_timec(cfg):
    """The real part of the absorber timec (DFT4He3d.f90:689-699) that
    he4g_create builds, float32 of shape (nz, ny, nx); the imaginary part is 1."""
    lib = abi.load()
    out = np.empty((cfg.nz, cfg.ny, cfg.nx), dtype=np.float32)
    rc = lib.he4g_build_timec(C.byref(cfg), out.ctypes.data_as(C.POINTER(C.c_float)))
    if rc:
        raise He4gError(rc, "build_timec")
    return out


def read_namelist_int(path, name):
    """he4g_read_namelist_int: an integer of a namelist file, or None."""
    lib = abi.load()
    v = C.c_int()
    rc = lib.he4g_read_namelist_int(str(path).encode(), name.encode(), C.byref(v))
    return int(v.value) if rc == 0 else None


def potion_table(cfg, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463):
    """The radial impurity table alone (potenimpini), for runs whose k-space
    tables are built on the device."""
    lib = abi.load()
    po = np.empty(cfg.npot)
    rc = lib.he4g_build_tables(C.byref(cfg), selec.encode(), r_cutoff, umax, None, None, None, abi.dptr(po))
    if rc:
        raise He4gError(rc, "build_tables")
    return {"fvlj4": None, "wcgk": None, "kalfs": None, "potion": po}


class Run:
    """One GPU-resident run (he4g_run). device_tables: build fvlj4, wcgk and
    kalfs on the device (he4g_create with NULL table pointers) instead of on
    the host; only the radial impurity table is built here."""

    def __init__(self, cfg, tables=None, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463, device_tables=False):
        self.lib = abi.load()
        self.cfg = cfg
        if tables is None:
            tables = (potion_table if device_tables else build_tables)(cfg, selec, r_cutoff, umax)
        self.tables = tables
        self.shape = (cfg.nz, cfg.ny, cfg.nx)
        h = C.c_void_p()
        t = self.tables

        def ptr(name):
            return abi.dptr(t[name]) if t.get(name) is not None else None

        rc = self.lib.he4g_create(C.byref(cfg), ptr("fvlj4"), ptr("wcgk"), ptr("kalfs"), abi.dptr(t["potion"]),
                                  C.byref(h))
        if rc:
            raise He4gError(rc, "he4g_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.he4g_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        if rc:
            msg = self.lib.he4g_last_error(self.h)
            raise He4gError(rc, msg.decode() if msg else "")

    # ---------------------------------------------------------------- state
    def set_state(self, psi, rimp, vimp):
        psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(self.shape)
        r = np.ascontiguousarray(rimp, dtype=np.float64)
        v = np.ascontiguousarray(vimp, dtype=np.float64)
        self._ck(self.lib.he4g_set_state(self.h, abi.dptr(psi), abi.dptr(r), abi.dptr(v)))

    # -------------------------------------------------- reference routines
    def potenimp(self, rimp):
        r = np.ascontiguousarray(rimp, dtype=np.float64)
        self._ck(self.lib.he4g_potenimp(self.h, abi.dptr(r)))

    def poten(self):
        self._ck(self.lib.he4g_poten(self.h))

    def forceimp(self, rimp=(0.0, 0.0, 0.0)):
        r = np.ascontiguousarray(rimp, dtype=np.float64)
        F = np.zeros(3)
        self._ck(self.lib.he4g_forceimp(self.h, abi.dptr(r), abi.dptr(F)))
        return F

    def steprk(self, deltat):
        self._ck(self.lib.he4g_steprk(self.h, deltat))

    def steppc(self, deltat):
        e = np.zeros(2)
        self._ck(self.lib.he4g_steppc(self.h, deltat, abi.dptr(e[:1]), abi.dptr(e[1:])))
        return float(e[0]), float(e[1])

    def step(self, nsteps=1):
        e = np.zeros(2)
        self._ck(self.lib.he4g_step(self.h, nsteps, abi.dptr(e[:1]), abi.dptr(e[1:])))
        return float(e[0]), float(e[1])

    def step_timed(self, nsteps):
        """he4g_step with CUDA events on the run's stream; returns device ms."""
        ms = np.zeros(1)
        self._ck(self.lib.he4g_step_timed(self.h, nsteps, abi.dptr(ms)))
        return float(ms[0])

    @property
    def launch_count(self):
        return int(self.lib.he4g_launch_count(self.h))

    def enable_graphs(self, on=True):
        self._ck(self.lib.he4g_enable_graphs(self.h, 1 if on else 0))

    def autotune(self, reps=5):
        """Time every FFT tile shape and engine on this run's buffers and keep
        the fastest.

        Returns (lpb_r2c, lpb_c2r, log2 cols y, log2 cols z, register-engine
        bits: 1 forward x, 2 inverse x, 4 y, 8 z)."""
        t = (C.c_int * NTILES)()
        self._ck(self.lib.he4g_autotune(self.h, reps, t))
        return tuple(t)

    @property
    def tiles(self):
        t = (C.c_int * NTILES)()
        self._ck(self.lib.he4g_get_tiles(self.h, t))
        return tuple(t)

    @tiles.setter
    def tiles(self, value):
        t = (C.c_int * NTILES)(*[int(v) for v in value])
        self._ck(self.lib.he4g_set_tiles(self.h, t))

    def energy(self):
        en = abi.Energies()
        self._ck(self.lib.he4g_energy(self.h, C.byref(en)))
        return en.as_dict()

    def r_cm(self, npart):
        cm = np.zeros(3)
        self._ck(self.lib.he4g_r_cm(self.h, float(npart), abi.dptr(cm)))
        return cm

    def observables(self, npart):
        o = abi.Obs()
        self._ck(self.lib.he4g_observables(self.h, float(npart), C.byref(o)))
        return {"npart": o.npart, "cm": list(o.cm), "ang": list(o.ang), "ang_im": list(o.ang_im),
                "r2": list(o.r2)}

    # ------------------------------------------------------------- readback
    @property
    def psi(self):
        out = np.empty(self.shape, dtype=np.complex128)
        self._ck(self.lib.he4g_get_psi(self.h, abi.dptr(out)))
        return out

    def get_psi_async(self, out):
        """Starts copying psi into `out` (a complex128 array of the grid's
        shape, pinned for the copy to overlap the next steps) and returns;
        wait_psi() waits for it. `out` must stay alive until then."""
        if out.dtype != np.complex128 or out.size != self.cfg.nx * self.cfg.ny * self.cfg.nz or \
                not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out: a contiguous complex128 array of nx*ny*nz values")
        self._ck(self.lib.he4g_get_psi_async(self.h, abi.dptr(out)))

    def wait_psi(self):
        self._ck(self.lib.he4g_wait_psi(self.h))

    @property
    def den(self):
        out = np.empty(self.shape)
        self._ck(self.lib.he4g_get_den(self.h, abi.dptr(out)))
        return out

    FIELDS = {"pot4": 0, "dencg": 1, "delj4": 2, "uimp": 3, "dxden": 4, "dyden": 5, "dzden": 6,
              "ualphas": 7, "denalf": 8}

    def field(self, name):
        out = np.empty(self.shape)
        self._ck(self.lib.he4g_get_field(self.h, self.FIELDS[name], abi.dptr(out)))
        return out

    def write_density(self, path, n4, time_ps=0.0, selec="Xe_He", r_cutoff=2.55, umax=2793.9365463):
        """The reference's restart/output file (printoutc.f90) of the current
        state: energies, observables, rimp, vimp and psi; readenc mode 2
        (and he4gpu.formats.read_density) read it back."""
        from . import formats
        e, o = self.energy(), self.observables(n4)
        r, v, _ = self.impurity()
        # the run's arrays are (nz, ny, nx) with x fastest; the file helpers
        # take (nx, ny, nz) arrays in Fortran order, the same memory
        formats.write_density(path, self.psi.transpose(2, 1, 0), r, v, self.cfg.xmax, self.cfg.ymax, self.cfg.zmax,
                              iteration=self.steps_taken, dtps=self.cfg.deltat * formats.PS_PER_KELVIN_UNIT,
                              time=time_ps, selec=selec, r_cutoff=r_cutoff, umax=umax, cm=o["cm"],
                              npart=o["npart"], energies=e, ang=o["ang"], r2=o["r2"])

    def health(self):
        """(code, message) of the run's checks after its queued work
        (he4g_health): code 0 when healthy; does not raise."""
        rc = self.lib.he4g_health(self.h)
        msg = self.lib.he4g_last_error(self.h)
        return rc, (msg.decode() if rc and msg else "")

    def save_snapshot(self):
        """The run's whole time-stepping state (he4g_save_snapshot) as a numpy
        uint8 array; load_snapshot restores it into a run of the same grid,
        box, core and form, which then continues bit for bit."""
        n = C.c_uint64()
        self._ck(self.lib.he4g_snapshot_bytes(self.h, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        self._ck(self.lib.he4g_save_snapshot(self.h, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf

    def load_snapshot(self, buf):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self._ck(self.lib.he4g_load_snapshot(self.h, buf.ctypes.data_as(C.c_void_p), buf.size))

    def read_state(self, path, mode=2):
        """set_state from a reference density / wave-function file (readenc
        modes 0, 2, 3); mode 0 densities become psi = sqrt(den)."""
        from . import formats
        d = formats.read_density(path, mode)
        if (d["nx"], d["ny"], d["nz"]) != (self.cfg.nx, self.cfg.ny, self.cfg.nz):
            raise He4gError(-1, f"{path}: grid {d['nx']}x{d['ny']}x{d['nz']} does not match the run")
        psi = d["psi"] if "psi" in d else np.sqrt(np.maximum(d["den"], 0.0)).astype(np.complex128)
        # (nx, ny, nz) in Fortran order -> the run's (nz, ny, nx), x fastest
        self.set_state(psi.transpose(2, 1, 0), d["rimp"], d.get("vimp", np.zeros(3)))
        return d

    def impurity(self):
        r, v, a = np.zeros(3), np.zeros(3), np.zeros(3)
        self._ck(self.lib.he4g_get_impurity(self.h, abi.dptr(r), abi.dptr(v), abi.dptr(a)))
        return r, v, a

    def set_timec(self, timec):
        """he4g_set_timec: the absorber from a complex128 (nz, ny, nx) array
        shaped like the driver's timec module array."""
        t = np.ascontiguousarray(timec, dtype=np.complex128).reshape(self.shape)
        self._ck(self.lib.he4g_set_timec(self.h, abi.dptr(t)))

    def set_uext(self, uext):
        """he4g_set_uext: the external potential of the energy (None: none)."""
        if uext is None:
            self._ck(self.lib.he4g_set_uext(self.h, None))
            return
        u = np.ascontiguousarray(uext, dtype=np.float64).reshape(self.shape)
        self._ck(self.lib.he4g_set_uext(self.h, abi.dptr(u)))

    def set_impurity(self, r, v, a):
        r, v, a = (np.ascontiguousarray(x, dtype=np.float64) for x in (r, v, a))
        self._ck(self.lib.he4g_set_impurity(self.h, abi.dptr(r), abi.dptr(v), abi.dptr(a)))

    def trajectory(self, cap=8192):
        rows = np.zeros((cap, 10))
        n = C.c_int()
        self._ck(self.lib.he4g_get_trajectory(self.h, abi.dptr(rows), cap, C.byref(n)))
        return rows[: n.value]

    @property
    def steps_taken(self):
        return self.lib.he4g_steps_taken(self.h)

    def enable_timing(self, on=True):
        self._ck(self.lib.he4g_enable_timing(self.h, 1 if on else 0))

    def kernel_times(self):
        cap = 32
        names = (C.c_char_p * cap)()
        ms = np.zeros(cap)
        launches = (C.c_int * cap)()
        k = self.lib.he4g_kernel_times(self.h, names, abi.dptr(ms), launches, cap)
        if k < 0:
            self._ck(k)
        return {names[i].decode(): (float(ms[i]), int(launches[i])) for i in range(k)}


def step_many(runs, nsteps):
    """he4g_step_many: advance several runs together (their kernels overlap)."""
    if not runs:
        return
    lib = runs[0].lib
    arr = (C.c_void_p * len(runs))(*[r.h.value if isinstance(r.h, C.c_void_p) else r.h for r in runs])
    rc = lib.he4g_step_many(arr, len(runs), nsteps)
    if rc:
        msgs = [r.lib.he4g_last_error(r.h) for r in runs]
        raise He4gError(rc, "; ".join(m.decode() for m in msgs if m))


class Batch:
    """he4g_batch: a fixed set of runs advanced together, one CUDA graph per
    batch step (every run's step in one graph launch)."""

    def __init__(self, runs):
        self.runs = list(runs)
        self.lib = abi.load()
        arr = (C.c_void_p * len(self.runs))(*[r.h.value if isinstance(r.h, C.c_void_p) else r.h for r in self.runs])
        h = C.c_void_p()
        rc = self.lib.he4g_batch_create(arr, len(self.runs), C.byref(h))
        if rc:
            raise He4gError(rc, "he4g_batch_create failed")
        self.h = h

    def step(self, nsteps):
        rc = self.lib.he4g_batch_step(self.h, nsteps)
        if rc:
            msgs = [r.lib.he4g_last_error(r.h) for r in self.runs if getattr(r, "h", None)]
            raise He4gError(rc, "; ".join(m.decode() for m in msgs if m))

    @property
    def graphs(self):
        return int(self.lib.he4g_batch_graphs(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.he4g_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
