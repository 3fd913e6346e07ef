"""GPU checks of the mixed-precision form (HE4G_PREC_MIXED): FP32 FFT
convolutions, stencils, H.psi and pointwise functional; FP64 psi accumulator,
norm and energy sums, force sum and impurity trajectory.

Its error against the FP64 oracle is that of FP32 fields (about 1e-7
relative per evaluation), so the tolerances here are FP32-scale: density and
energies to 1e-5 relative after a few tens of steps, the impurity position to
1e-8. Drift statements over long runs come from he4gpu/drift.py; the
10^4-step record of the 256^3 collision is tests/records/drift_mixed_he5000_xe_256.json.
"""
import numpy as np
import pytest

from helpers import gpu_run, make_case, oracle_run, rel, rel_field, rel_vec

pytestmark = pytest.mark.gpu

MIXED = 1


@pytest.mark.parametrize("case,nsteps", [("he100_xe_32", 20), ("he300_ar_48", 12), ("he200_xe_40x48x64", 10)])
def test_mixed_tracks_fp64_oracle(case, nsteps):
    cfg, tk, psi, r, v, meta = make_case(case, precision=MIXED)
    g = gpu_run(cfg, tk, psi, r, v)
    cfg64, *_ = make_case(case)
    o = oracle_run(cfg64, tk, psi, r, v)
    assert rel_field(g.field("pot4"), o.field("pot4")) < 1e-5
    assert rel_field(g.field("dencg"), o.field("dencg")) < 1e-5
    g.step(nsteps)
    o.step(nsteps)
    assert rel_field(g.den, o.den) < 1e-5
    assert rel_field(g.psi, o.psi) < 1e-5
    rg, vg, ag = g.impurity()
    ro, vo, ao = o.impurity()
    assert rel_vec(rg, ro) < 1e-8 and rel_vec(vg, vo) < 1e-6 and rel_vec(ag, ao) < 1e-3
    eg, eo = g.energy(), o.energy()
    for k in ("etot", "etot4", "ekin4", "elj4", "ecor4", "ekinx", "eHeX"):
        assert abs(eg[k] - eo[k]) <= 1e-5 * max(abs(eo[k]), 1.0), (k, eg[k], eo[k])
    assert rel(g.observables(meta["n4"])["npart"], o.observables(meta["n4"])["npart"]) < 1e-6
    g.close()
    o.close()


def test_mixed_conserves_norm_and_energy_without_absorber():
    """Without the absorber the mixed form conserves the norm and the energy as
    well as the FP64 form does, to FP32 noise."""
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=MIXED, lambdah=0.0)
    g = gpu_run(cfg, tk, psi, r, v)
    cfg64, *_ = make_case("he100_xe_32", lambdah=0.0)
    d = gpu_run(cfg64, tk, psi, r, v)
    n0 = g.observables(meta["n4"])["npart"]
    e0 = g.energy()["etot"]
    f0 = d.energy()["etot"]
    g.step(200)
    d.step(200)
    n1 = g.observables(meta["n4"])["npart"]
    e1 = g.energy()["etot"]
    f1 = d.energy()["etot"]
    assert abs(n1 - n0) / n0 < 1e-7
    # the mixed form's energy drift stays within 1e-6 of the FP64 form's
    assert abs((e1 - e0) - (f1 - f0)) / abs(f0) < 1e-6


def test_mixed_otc_alpha_s():
    cfg, tk, psi, r, v, meta = make_case("he100_xe_32", precision=MIXED, core=1, lsolid=0, hcg=2.190323)
    g = gpu_run(cfg, tk, psi, r, v)
    cfg64, *_ = make_case("he100_xe_32", core=1, lsolid=0, hcg=2.190323)
    o = oracle_run(cfg64, tk, psi, r, v)
    for name in ("ualphas", "pot4", "denalf"):
        assert rel_field(g.field(name), o.field(name)) < 1e-4, name
    eg, eo = g.energy(), o.energy()
    assert abs(eg["ealphas"] - eo["ealphas"]) <= 1e-4 * abs(eo["ealphas"])
    g.step(6)
    o.step(6)
    assert rel_field(g.den, o.den) < 1e-5
