"""Batched ensembles and the serving loop (include/mhh_batch.h).

Every model in an ensemble or a job in the server runs the same kernels with
the same arguments as alone, so its fields must be bitwise identical to a run
of the same model alone, in every mode.
"""
import numpy as np
import pytest

from microhh_gb300 import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mhh():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import microhh_gb300
    microhh_gb300.load()
    return microhh_gb300


def members():
    # Uneven sizes, each with its own seed and surface flux.
    return [
        cases.drycbl(32, 32, 32, 3200., 3200., 3200., seed=51, sbot=0.08, noise_z=800.),
        cases.drycbl(48, 48, 64, 4800., 4800., 4000., seed=52, sbot=0.20, noise_z=800.),
        cases.drycbl(40, 24, 20, 4000., 2400., 2000., seed=53, sbot=0.12, noise_z=600.),
        cases.drycbl(64, 64, 40, 6400., 6400., 3200., seed=54, sbot=0.16, noise_z=800.),
    ]


def alone(mhh, case, nsteps):
    m = mhh.Model(case, precision=mhh.FP32)
    m.run_steps(nsteps)
    out = {n: m.get(n) for n in case.prognostic_names()}
    m.close()
    return out


@pytest.mark.parametrize("mode", [0, 1, 2, 3], ids=["sequential", "streams", "graphs", "batched"])
def test_ensemble_identical_to_alone(mhh, mode):
    cs = members()
    ref = [alone(mhh, c, 4) for c in cs]
    models = [mhh.Model(c, precision=mhh.FP32) for c in cs]
    ens = mhh.Ensemble(models)
    n0 = mhh.launch_count()
    ens.run_steps(1, mode)
    ens.run_steps(3, mode)
    ens.synchronize()
    assert mhh.launch_count() > n0
    for c, m, r in zip(cs, models, ref):
        for n in c.prognostic_names():
            assert np.array_equal(m.get(n), r[n]), (c.name, n, mode)
    ens.close()


def test_batched_launches_scale_with_stages(mhh):
    """Batched mode launches one kernel per stage for all members of one grid
    size, so the launches of a step grow with the number of distinct sizes,
    not with the number of members: doubling the members (same sizes, other
    states) keeps the count, while the members' own graphs double it."""
    def launches_per_step(cs, mode):
        models = [mhh.Model(c, precision=mhh.FP32) for c in cs]
        ens = mhh.Ensemble(models)
        ens.run_steps(2, mode)
        ens.synchronize()
        n0 = mhh.launch_count()
        ens.run_steps(2, mode)
        ens.synchronize()
        n = (mhh.launch_count() - n0) / 2
        ens.close()
        for m in models:
            m.close()
        return n
    once = members()
    twice = members() + members()
    for q, c in enumerate(twice[4:]):
        c.fields["th"] = c.fields["th"] + 0.01 * (q + 1)
    batch_once = launches_per_step(once, mhh.ENS_BATCHED)
    batch_twice = launches_per_step(twice, mhh.ENS_BATCHED)
    graph_once = launches_per_step(once, mhh.ENS_GRAPHS)
    graph_twice = launches_per_step(twice, mhh.ENS_GRAPHS)
    assert batch_twice == batch_once, (batch_once, batch_twice)
    assert graph_twice == 2 * graph_once, (graph_once, graph_twice)
    assert batch_twice <= graph_twice / 2, (batch_twice, graph_twice)


def test_ensemble_autotune_keeps_state_and_parity(mhh):
    cs = members()[:2]
    models = [mhh.Model(c, precision=mhh.FP32) for c in cs]
    ens = mhh.Ensemble(models)
    before = [{n: m.get(n) for n in c.prognostic_names()} for c, m in zip(cs, models)]
    report = ens.autotune()
    assert "32x32x32" in report and "48x48x64" in report
    for c, m, b in zip(cs, models, before):
        for n in c.prognostic_names():
            assert np.array_equal(m.get(n), b[n])
    ens.run_steps(3, mhh.ENS_GRAPHS)
    ens.synchronize()
    # The tuned kernel variants differ from the defaults by float round-off
    # only (held to the FP32 form's tolerance, relative L2).
    for c, m in zip(cs, models):
        r = alone(mhh, c, 3)
        for n in ("u", "v", "w"):
            err = np.linalg.norm(m.get(n) - r[n]) / np.linalg.norm(r[n])
            assert err <= 2e-3, (c.name, n, err)
        # theta ~ 300 K carries 3e-5 K per float ulp; three steps through
        # differently rounded kernels stay within a few ulps.
        assert np.abs(m.get("th") - r["th"]).max() <= 5e-4
    ens.close()


def test_server_results_same_alone_and_in_mix(mhh):
    cs = members()
    shapes = [mhh.Model(c, precision=mhh.FP32).shape for c in cs[:1]]
    steps = [5, 3, 4, 2]
    srv = mhh.Server(budget_bytes=8e9, max_active=4)
    ids = [srv.submit(c, n, arrival=0.002 * q, keep=True) for q, (c, n) in enumerate(zip(cs, steps))]
    srv.run(mhh.SERVE_CONTINUOUS)
    mixed = {n: srv.result(ids[0], n, shapes[0]) for n in cs[0].prognostic_names()}
    # FIFO on the same server: the same results.
    srv.run(mhh.SERVE_FIFO)
    for n in cs[0].prognostic_names():
        assert np.array_equal(srv.result(ids[0], n, shapes[0]), mixed[n]), n
    for j in ids:
        a, ad, f = srv.times(j)
        assert 0 <= a <= ad + 1e-3 and ad <= f
    srv.close()
    # The job alone in its own server, and the plain model run.
    solo = mhh.Server(budget_bytes=8e9, max_active=1)
    j = solo.submit(cs[0], steps[0], keep=True)
    solo.run(mhh.SERVE_CONTINUOUS)
    ref = alone(mhh, cs[0], steps[0])
    for n in cs[0].prognostic_names():
        got = solo.result(j, n, shapes[0])
        assert np.array_equal(got, mixed[n]), n
        assert np.array_equal(got, ref[n]), n
    solo.close()


def test_server_admission_respects_budget(mhh):
    cs = members()
    srv = mhh.Server(budget_bytes=1.0, max_active=4)   # below any job: one at a time
    ids = [srv.submit(c, 2) for c in cs]
    srv.run(mhh.SERVE_CONTINUOUS)
    spans = sorted(srv.times(j)[1:] for j in ids)
    for (a0, f0), (a1, f1) in zip(spans, spans[1:]):
        assert a1 >= f0 - 1e-6, (spans,)
    srv.close()
