"""Shared set-up of matching GPU and oracle runs for the parity tests."""
import numpy as np


def make_case(case, seed=0, extents=None, **over):
    """Configuration, table keys, state and metadata of a named collision
    workload; extents = (xmax, ymax, zmax) replaces the box half-extents before
    the defaults that depend on them (the impurity table spacing) are set."""
    import he4gpu
    psi, r, v, meta = he4gpu.collision_case(case, seed=seed)
    kw, tk = he4gpu.config_for_case(meta)
    kw.update(over)
    ext = extents or (meta["xmax"], meta["ymax"], meta["zmax"])
    cfg = he4gpu.default_config(meta["nx"], meta["ny"], meta["nz"], *ext, **kw)
    return cfg, tk, psi, r, v, meta


def gpu_run(cfg, tk, psi, r, v):
    import he4gpu
    run = he4gpu.Run(cfg, selec=tk["selec"], r_cutoff=tk["r_cutoff"], umax=tk["umax"])
    run.set_state(psi, r, v)
    return run


def oracle_run(cfg, tk, psi, r, v):
    from oracle import oracle
    tabs = oracle.build_tables(cfg, tk["selec"], tk["r_cutoff"], tk["umax"])
    o = oracle.OracleRun(cfg, tabs)
    o.set_state(psi, r, v)
    return o


def rel_field(a, b):
    """max |a - b| / max |b|"""
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel_vec(a, b):
    """max |a - b| / max |b| for small vectors (components that vanish by
    symmetry, such as an impurity's y coordinate, are judged on the vector's
    scale)."""
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))
