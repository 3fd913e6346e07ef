"""ctypes declarations of include/he4g.h and the loader of libhe4g.so.

The library is the only compute path: `load()` raises when it is missing or
was built without a symbol the header declares, and there is no fallback.
"""
import ctypes as C
import os

from . import build as _build

HE4G_OK = 0
HE4G_EINVAL = -1
HE4G_ENOMEM = -2
HE4G_ECUDA = -3
HE4G_EDENSITY = -4
HE4G_ENAN = -5
HE4G_ETABLE = -6
HE4G_ESTATE = -7

CORE_OT = 0
CORE_OTC = 1
PREC_FP64 = 0
PREC_MIXED = 1
PREC_DF64 = 2

ERRORS = {
    HE4G_EINVAL: "invalid argument",
    HE4G_ENOMEM: "device allocation failed",
    HE4G_ECUDA: "CUDA error",
    HE4G_EDENSITY: "density not > 0",
    HE4G_ENAN: "non-finite state",
    HE4G_ETABLE: "impurity beyond the potential table",
    HE4G_ESTATE: "call out of order",
}


class Config(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("npd", C.c_int32), ("icon", C.c_int32), ("core", C.c_int32),
        ("lsolid", C.c_int32), ("lrk", C.c_int32), ("precision", C.c_int32),
        ("npot", C.c_int32),
        ("xmax", C.c_double), ("ymax", C.c_double), ("zmax", C.c_double),
        ("deltat", C.c_double),
        ("cp4", C.c_double), ("cpp4", C.c_double), ("h2o2m4", C.c_double),
        ("alphas", C.c_double), ("l_alpha", C.c_double), ("den0s", C.c_double),
        ("c_solid", C.c_double), ("beta_solid", C.c_double), ("den_m", C.c_double),
        ("eps4", C.c_double), ("sigma4", C.c_double), ("h4", C.c_double), ("hcg", C.c_double),
        ("lambdah", C.c_double), ("txmean", C.c_double), ("txsurf", C.c_double),
        ("tymean", C.c_double), ("tysurf", C.c_double), ("tzmean", C.c_double),
        ("tzsurf", C.c_double),
        ("mimpur", C.c_double), ("delinter", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Energies(C.Structure):
    _fields_ = [(k, C.c_double) for k in
                ("etot4", "ekin4", "elj4", "ecor4", "ealphas", "esolid", "eext",
                 "ekinx", "eHeX", "eimpu", "etot")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Obs(C.Structure):
    _fields_ = [("npart", C.c_double), ("cm", C.c_double * 3), ("ang", C.c_double * 3),
                ("ang_im", C.c_double * 3), ("r2", C.c_double * 3)]


def reference_defaults(nx, ny, nz, xmax, ymax, zmax):
    """The values he4g_default_config fills, computed here without loading
    libhe4g.so, for processes that must not map the GPU library (the CPU
    timing of the oracle). The module defaults of modules.f90 (he4 :138-148,
    lenard4 :209-212, deriva :27-33), the absorber of the shipped input
    (input_files/xe-he1000-hoc-200mps.input:2-4), h_cg = 1.065 h4 for
    lsolid (DFT4He3d.f90:579-586) and the table size of potenimpini.f90:13-16.
    tests/test_abi.py holds it equal to the library's, field by field."""
    c = Config()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.npd, c.icon, c.core, c.lsolid, c.lrk, c.precision = 13, 13, CORE_OT, 1, 0, PREC_FP64
    c.xmax, c.ymax, c.zmax, c.deltat = xmax, ymax, zmax, 0.0
    c.cp4, c.cpp4, c.h2o2m4 = -2.41186e4, 1.85850e6, 6.05969638298
    c.alphas, c.l_alpha, c.den0s = 54.31, 1.0, 0.04
    c.c_solid, c.beta_solid, c.den_m = 3.1577504e4, 40.0, 0.37
    c.eps4, c.sigma4, c.h4 = 10.22, 2.556, 2.190323
    c.hcg = 2.190323 * 1.065
    c.lambdah, c.txmean, c.txsurf, c.tymean, c.tysurf, c.tzmean, c.tzsurf = 2.0, 1000.0, 2.0, 1000.0, 2.0, 49.2, 2.0
    c.mimpur = 131.29
    c.npot = 100 * max(nx, ny, nz) + 1
    c.delinter = 4.0 * max(xmax, ymax, zmax) / float(c.npot - 1)
    return c


_D = C.POINTER(C.c_double)
_P = C.c_void_p

# name -> (restype, argtypes); every function include/he4g.h declares
SIGNATURES = {
    "he4g_default_config": (None, [C.POINTER(Config), C.c_int, C.c_int, C.c_int,
                                   C.c_double, C.c_double, C.c_double]),
    "he4g_build_tables": (C.c_int, [C.POINTER(Config), C.c_char_p, C.c_double, C.c_double,
                                    _D, _D, _D, _D]),
    "he4g_create": (C.c_int, [C.POINTER(Config), _D, _D, _D, _D, C.POINTER(_P)]),
    "he4g_destroy": (None, [_P]),
    "he4g_last_error": (C.c_char_p, [_P]),
    "he4g_set_state": (C.c_int, [_P, _D, _D, _D]),
    "he4g_potenimp": (C.c_int, [_P, _D]),
    "he4g_poten": (C.c_int, [_P]),
    "he4g_forceimp": (C.c_int, [_P, _D, _D]),
    "he4g_steprk": (C.c_int, [_P, C.c_double]),
    "he4g_steppc": (C.c_int, [_P, C.c_double, _D, _D]),
    "he4g_energy": (C.c_int, [_P, C.POINTER(Energies)]),
    "he4g_r_cm": (C.c_int, [_P, C.c_double, _D]),
    "he4g_observables": (C.c_int, [_P, C.c_double, C.POINTER(Obs)]),
    "he4g_step": (C.c_int, [_P, C.c_int, _D, _D]),
    "he4g_get_trajectory": (C.c_int, [_P, _D, C.c_int, C.POINTER(C.c_int)]),
    "he4g_get_psi": (C.c_int, [_P, _D]),
    "he4g_get_psi_async": (C.c_int, [_P, _D]),
    "he4g_wait_psi": (C.c_int, [_P]),
    "he4g_get_den": (C.c_int, [_P, _D]),
    "he4g_get_field": (C.c_int, [_P, C.c_int, _D]),
    "he4g_get_impurity": (C.c_int, [_P, _D, _D, _D]),
    "he4g_set_impurity": (C.c_int, [_P, _D, _D, _D]),
    "he4g_step_timed": (C.c_int, [_P, C.c_int, _D]),
    "he4g_forceimp_noalloc": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_double, _P, _P]),
    "he4g_launch_count": (C.c_longlong, [_P]),
    "he4g_enable_graphs": (C.c_int, [_P, C.c_int]),
    "he4g_footprint": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_uint64)]),
    "he4g_step_many": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int]),
    "he4g_autotune": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int)]),
    "he4g_get_tiles": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "he4g_set_tiles": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "he4g_steps_taken": (C.c_int, [_P]),
    "he4g_health": (C.c_int, [_P]),
    "he4g_snapshot_bytes": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "he4g_save_snapshot": (C.c_int, [_P, _P, C.c_uint64]),
    "he4g_load_snapshot": (C.c_int, [_P, _P, C.c_uint64]),
    "he4g_kernel_times": (C.c_int, [_P, C.POINTER(C.c_char_p), _D, C.POINTER(C.c_int), C.c_int]),
    "he4g_enable_timing": (C.c_int, [_P, C.c_int]),
    "he4g_set_timec": (C.c_int, [_P, _D]),
    "he4g_set_uext": (C.c_int, [_P, _D]),
    "he4g_build_uext": (C.c_int, [C.POINTER(Config), C.c_int, C.c_double, _D]),
    "he4g_build_timec": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_float)]),
    "he4g_read_namelist_int": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_int)]),
    "he4g_batch_create": (C.c_int, [C.POINTER(_P), C.c_int, C.POINTER(_P)]),
    "he4g_batch_step": (C.c_int, [_P, C.c_int]),
    "he4g_batch_graphs": (C.c_int, [_P]),
    "he4g_batch_destroy": (None, [_P]),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads libhe4g.so (building it first when missing); raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with he4gpu.build.build()")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError when the symbol is missing
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a):
    """double* of a C-contiguous float64 / complex128 numpy array."""
    return a.ctypes.data_as(_D)
