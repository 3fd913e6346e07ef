"""The serving loop's host logic (he4gpu/serve.py: admission by device
footprint, continuous batching in chunks, eviction of failed jobs, the
report) on the CPU, with the GPU calls replaced by fakes that count steps.
The GPU tests (tests/test_gpu_serve.py) run the same loop on real runs."""
import numpy as np
import pytest

from he4gpu import He4gError, serve


class FakeRun:
    def __init__(self, meta):
        self.meta = meta
        self.steps = 0
        self.closed = False
        self.code = 0

    def set_state(self, psi, r, v):
        if self.meta.get("bad_state"):
            raise He4gError(-4, "density not > 0 after a Runge-Kutta stage")

    def health(self):
        return (self.code, "density not > 0" if self.code else "")

    def close(self):
        self.closed = True


@pytest.fixture
def fakes(monkeypatch):
    made = []
    calls = []

    def make_run(meta, precision, **kw):
        r = FakeRun(meta)
        made.append(r)
        return r, type("Cfg", (), {"nx": meta["nx"], "ny": meta["ny"], "nz": meta["nz"]})()

    def step_many(runs, k):
        fails = any(r.meta.get("fail_at") is not None and r.steps < r.meta["fail_at"] <= r.steps + k for r in runs)
        calls.append((len(runs), k, fails))
        assert all(not r.closed for r in runs)
        failed = False
        for r in runs:
            fail_at = r.meta.get("fail_at")
            if fail_at is not None and r.steps < fail_at <= r.steps + k:
                r.code = -4  # this run stops at its failing step; the others take their k steps
                r.steps = fail_at
                failed = True
            else:
                r.steps += k
        if failed:
            raise He4gError(-4, "density not > 0")

    monkeypatch.setattr(serve, "make_run", make_run)
    monkeypatch.setattr(serve, "step_many", step_many)
    monkeypatch.setattr(serve, "job_config", lambda meta, precision: meta)
    monkeypatch.setattr(serve, "footprint", lambda meta: meta["bytes"])
    monkeypatch.setattr(serve, "final_state", lambda run, meta: {"steps": run.steps})
    return made, calls


def job(steps, nbytes=10, **kw):
    return dict(nx=32, ny=32, nz=32, steps=steps, bytes=nbytes, n4=100, **kw)


def no_state(meta):
    return None, None, None


def test_every_job_runs_its_steps_within_the_memory_budget(fakes):
    made, calls = fakes
    stream = [(0.0, job(s)) for s in (40, 16, 70, 33, 16, 5)]
    rep, _ = serve.serve(stream, hbm_budget=35, chunk=16, state_fn=no_state, keep_results=())
    assert rep["jobs"] == 6 and rep["failed"] == []
    # three 10-byte jobs fit a 35-byte budget at a time
    assert rep["max_resident"] == 3 and max(n for n, _, _ in calls) == 3
    assert {j: f["steps"] for j, f in rep["finals"].items()} == {i: m["steps"] for i, (_, m) in enumerate(stream)}
    # a chunk never takes a resident job past its last step
    assert all(k <= 16 for _, k, _ in calls)
    assert all(r.closed for r in made)


def test_a_job_larger_than_the_budget_runs_alone(fakes):
    made, calls = fakes
    stream = [(0.0, job(20, nbytes=50)), (0.0, job(20, nbytes=10))]
    rep, _ = serve.serve(stream, hbm_budget=35, chunk=8, state_fn=no_state, keep_results=())
    assert rep["jobs"] == 2 and rep["max_resident"] == 1
    assert all(n == 1 for n, _, _ in calls)


def test_failed_jobs_are_evicted_and_the_others_finish(fakes):
    made, calls = fakes
    stream = [(0.0, job(48)), (0.0, job(48, fail_at=20)), (0.0, job(48, bad_state=True)), (0.0, job(30))]
    rep, _ = serve.serve(stream, hbm_budget=100, chunk=16, state_fn=no_state, keep_results=())
    assert sorted(f["id"] for f in rep["failed"]) == [1, 2]
    assert rep["jobs"] == 2 and sorted(rep["finals"]) == [0, 3]
    assert rep["finals"][0]["steps"] == 48 and rep["finals"][3]["steps"] == 30
    # the failing run stopped at its step and left; the rejected one never stepped
    assert made[1].closed and made[1].steps == 20 and made[2].steps == 0
    # after the failing chunk the loop went on with the two healthy jobs only
    i = next(n for n, c in enumerate(calls) if c[2])
    assert calls[i][0] == 3 and all(n <= 2 for n, _, _ in calls[i + 1:])


def test_the_report_counts_grid_point_updates(fakes):
    made, calls = fakes
    stream = [(0.0, job(10)), (0.0, job(10))]
    rep, _ = serve.serve(stream, hbm_budget=100, chunk=4, state_fn=no_state, keep_results=())
    assert rep["jobs"] == 2
    assert rep["grid_point_updates_per_s"] * rep["makespan_s"] == pytest.approx(2 * 10 * 32 ** 3)
    assert np.isfinite(rep["step_latency_ms_p99"]) and rep["precision"] == "mixed"
