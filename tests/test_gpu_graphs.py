"""CUDA-graph replay of plain steps (stro_sim_set_graphs).

Past the ramp, stro_sim_run and stro_sim_run_sampled replay captured graphs of
the same launches they would make one by one. The DDFs must be bitwise those
of step-by-step launching and of the oracle, for every kernel path, across
property changes between runs (a changed setting must not replay a stale
graph) and across the ramp's end."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _channel(sg, gpu, precision, **kw):
    nx, ny, nz = 70, 22, 3
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = sg.Cell.solid
    fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = sg.Cell.inflow
    s = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=1.6, omegaMinus=1.3,
                      uin=0.05, rampSteps=kw.pop("rampSteps", 40), wantsForces=True,
                      flags=fl.reshape(-1), **kw)
    s.setSolidFractions(np.tile(sg.diskSolidFractions(nx, ny, 15.5, 10.5, 4.0), nz))
    s.sponge = (50.0, 15.0, 0.9)
    return s


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
@pytest.mark.parametrize("split", [True, False])
def test_graph_replay_equals_step_by_step(gpu, precision, split):
    import strouhal_gb300 as sg

    a, b = _channel(sg, gpu, precision), _channel(sg, gpu, precision)
    a.setBlockSplit(split)
    b.setBlockSplit(split)
    b.setGraphs(False)
    for steps in (150, 3, 97, 64):  # across the ramp's end, odd starts, a short run
        a.run(steps)
        b.run(steps)
        assert a.stepsDone == b.stepsDone
        assert a.stateDigest == b.stateDigest, (steps, a.stepsDone)
    # a changed setting is a different graph, not a stale one
    a.omega = b.omega = 1.7
    a.force = b.force = (1e-5, 0.0, 0.0)
    for _ in range(2):
        a.run(80)
        b.run(80)
        assert a.stateDigest == b.stateDigest
    a.close()
    b.close()


@pytest.mark.parametrize("variant,kind", [(0, "fp32"), (1, "fp16s"), (3, "fp32"), (2, "fp32")])
def test_graph_replay_periodic_variants(gpu, variant, kind):
    import strouhal_gb300 as sg

    sims = []
    for graphs in (True, False):
        s = sg.Simulation(gpu, precision=kind, nx=128, ny=16, nz=8, omega=1.8)
        s.initField(2, 0.05)
        s.variant = variant
        if variant == 3:
            s.block = (64, 2)
        s.setGraphs(graphs)
        sims.append(s)
    for steps in (200, 66):
        for s in sims:
            s.run(steps)
        assert sims[0].stateDigest == sims[1].stateDigest
    assert sims[0].lastPath == sims[1].lastPath
    for s in sims:
        s.close()


def test_graph_replay_matches_oracle(gpu, oracle):
    import strouhal_gb300 as sg

    po = oracle
    nx, ny, nz = 40, 18, 3
    fl = np.zeros((nz, ny, nx), np.uint8)
    fl[:, 0, :] = fl[:, -1, :] = po.SOLID
    fl[:, 1:-1, 0] = fl[:, 1:-1, -1] = po.INFLOW
    kw = dict(omega=1.55, omegaMinus=1.2, uin=0.04, rampSteps=20, force=(2e-5, 0.0, 0.0))
    g = sg.Simulation(gpu, precision="fp32", nx=nx, ny=ny, nz=nz, flags=fl.reshape(-1), **kw)
    o = po.OracleSim(nx, ny, nz, flags=fl.reshape(-1), kind=0, **kw)
    g.run(150)
    o.run(150)
    assert np.array_equal(g.downloadState(), o.f)
    g.close()


def test_graph_replay_in_sampled_runs(gpu):
    from strouhal_gb300 import credibility as cr

    case = cr.StreetLadder()
    a, b = case.variant(gpu, 8, 1.0), case.variant(gpu, 8, 1.0)
    a.sim.rampSteps = b.sim.rampSteps = 100
    b.sim.setGraphs(False)
    fa, ta = a.sim.runSampled(300, 400, 26, *a.box)
    fb, tb = b.sim.runSampled(300, 400, 26, *b.box)
    assert np.array_equal(ta, tb)
    assert np.array_equal(fa, fb)
    assert a.sim.stateDigest == b.sim.stateDigest
    a.sim.close()
    b.sim.close()
