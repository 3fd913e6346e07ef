"""GPU check of the serving loop (he4gpu.serve) on a small stream: five jobs
on 32^3 and 48^3 grids arrive while others run, the HBM budget admits at most
two at a time (admission by he4g_footprint, eviction on completion), every
job's result in the mix equals its result alone bit for bit, and every job's
final state in the mixed form stays close to its plain-FP64 twin served one
job at a time: the norm within 1e-8, the total energy within 1e-5 of the
job's energy scale (the sum of its components' magnitudes).

The energy bar is taken on the job's energy scale because the total energy
is a difference of large components: the mixed form's FP32 fields put about
1e-7 relative error into each component, and for these toy droplets, which
fill their small boxes, |dE/E| reached 3.5e-4 on one job while every norm
stayed within 1e-9. The |dE/E| < 1e-6 bar of the serving workload is checked
on its own droplets: the 10^4-step record
tests/records/drift_mixed_he5000_xe_256.json and the serve tool's per-job
report."""
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    from he4gpu.initial import make_meta
    jobs = []
    spec = [(32, 100, "Xe", 12), (48, 300, "Ar", 9), (32, 150, "Ar", 14), (48, 200, "Xe", 10), (32, 120, "Xe", 8)]
    for i, (g, n4, imp, steps) in enumerate(spec):
        h = 0.8 if g == 32 else 0.6
        meta = make_meta(g, h, n4, imp, 0.3, 3.0, steps=steps, gap=2.0, seed=100 + i)
        jobs.append((0.05 * i, meta))
    return jobs


def test_serving_loop_admits_evicts_and_matches_runs_alone():
    import he4gpu
    from he4gpu import serve as S
    stream = _stream()
    need = max(he4gpu.footprint(S.job_config(m, S.MIXED)) for _, m in stream)
    rep, kept = S.serve(stream, 2 * need, chunk=4, keep_results=tuple(range(len(stream))))
    assert rep["jobs"] == len(stream)
    assert 1 <= rep["max_resident"] <= 2
    check = S.alone_vs_mix(stream, kept)
    assert all(v["identical"] for v in check.values()), check
    base = S.one_at_a_time_measured(stream)
    assert base["jobs"] == len(stream)
    drift = S.compare_finals(rep["finals"], base["finals"])
    assert drift["jobs_compared"] == len(stream)
    assert drift["dE_over_scale_max"] < 1e-5 and drift["norm_rel_max"] < 1e-8, drift


def test_a_failing_job_is_evicted_and_the_others_finish():
    """Host-side fault injection through the state upload: one job's psi has
    a slab of exact zeros deeper than the stencil, so its density check fails
    in its first Runge-Kutta stage (steprk.f90:89-92). The loop evicts that
    job with HE4G_EDENSITY and its memory; the other jobs, which shared the
    GPU with it, finish with the results they give alone."""
    import he4gpu
    from he4gpu import serve as S
    from he4gpu.initial import state_for
    stream = _stream()[:4]
    bad_meta = stream[1][1]

    def state_fn(meta):
        psi, r, v = state_for(meta)
        if meta is bad_meta:
            psi = psi.copy()
            psi[0:8, :, :] = 0.0
        return psi, r, v

    need = max(he4gpu.footprint(S.job_config(m, S.MIXED)) for _, m in stream)
    rep, kept = S.serve(stream, 2 * need, chunk=4, keep_results=(0, 2, 3), state_fn=state_fn)
    assert [f["id"] for f in rep["failed"]] == [1], rep["failed"]
    assert rep["failed"][0]["code"] == he4gpu.abi.HE4G_EDENSITY
    assert rep["jobs"] == 3
    check = S.alone_vs_mix(stream, kept)
    assert all(v["identical"] for v in check.values()), check
