"""Allocation-free observables (stro_observables_noalloc) against the allocating
entry points (stro_sim_kinetic_energy / stro_sim_dissipation).

Some callers cannot let the library allocate device memory while they step a
lattice: a framework whose own caching allocator has reserved the GPU's
memory, a real-time loop that cannot take the device synchronisation a
cudaMalloc may cause, or code running while a stream is captured. They hold
the DDF state in buffers they own and call the allocation-free entry point.
Here torch stands in for such a caller's allocator (the test owns the device
buffers). The file is collected last, so a failure here never hides another.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry(sg):
    fn = sg.lib().stro_observables_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                   ctypes.c_int32, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_float,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_noalloc_observables_match_allocating_entry_point(precision):
    torch = pytest.importorskip("torch")
    import strouhal_gb300 as sg

    fn = _entry(sg)
    gpu = sg.GPU(0)
    nx, ny, nz = 48, 40, 12
    flags = np.zeros((nz, ny, nx), np.uint8)
    flags[:, :, 0] = flags[:, :, -1] = flags[:, 0, :] = sg.Cell.solid
    flags[:, -1, :] = sg.Cell.lid
    force = (2e-6, -1e-6, 0.0)
    omega = 1.7
    sim = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=omega,
                        lid=(0.05, 0.0, 0.0), force=force, flags=flags.reshape(-1))
    sim.initField(2, 0.04)
    cells = torch.from_numpy(flags.reshape(-1).copy()).cuda()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    f3 = (ctypes.c_float * 3)(*force)
    prec = 0 if precision == "fp32" else 1
    for call in range(2):  # two calls in a row, each on a new state
        sim.run(6)
        state = torch.from_numpy(sim.downloadState()).cuda()  # canonical planes, stride N
        out.fill_(-1.0)
        rc = fn(state.data_ptr(), prec, nx, ny, nz, nx * ny * nz, cells.data_ptr(),
                omega, f3, out.data_ptr(), None)
        assert rc == 0, sg.lib().stro_last_error()
        torch.cuda.synchronize()
        ke, diss = out.cpu().numpy()
        assert np.isclose(ke, sim.kineticEnergySum(), rtol=1e-12, atol=0), (call, ke)
        assert np.isclose(diss, sim.dissipationSum(), rtol=1e-12, atol=0), (call, diss)
    # the same state in planes padded past N (a caller's own aligned layout)
    N = nx * ny * nz
    stride = N + 96
    padded = torch.full((19, stride), float("nan"), dtype=state.dtype, device="cuda")
    padded[:, :N] = state
    out.fill_(-1.0)
    rc = fn(padded.data_ptr(), prec, nx, ny, nz, stride, cells.data_ptr(), omega, f3,
            out.data_ptr(), None)
    assert rc == 0, sg.lib().stro_last_error()
    torch.cuda.synchronize()
    ke, diss = out.cpu().numpy()
    assert np.isclose(ke, sim.kineticEnergySum(), rtol=1e-12, atol=0), ke
    assert np.isclose(diss, sim.dissipationSum(), rtol=1e-12, atol=0), diss
    # refusals: sizes beyond what the entry point accepts, a plane stride below N,
    # a missing state or output pointer, and omega outside (0, 2) or NaN
    bad = [
        (state.data_ptr(), 2048, 2048, 1024, 1 << 33, omega, out.data_ptr()),
        (state.data_ptr(), nx, ny, nz, N - 1, omega, out.data_ptr()),
        (None, nx, ny, nz, N, omega, out.data_ptr()),
        (state.data_ptr(), nx, ny, nz, N, omega, None),
        (state.data_ptr(), nx, ny, nz, N, 0.0, out.data_ptr()),
        (state.data_ptr(), nx, ny, nz, N, 2.5, out.data_ptr()),
        (state.data_ptr(), nx, ny, nz, N, float("nan"), out.data_ptr()),
    ]
    for ptr, a, b, c, st, om, o in bad:
        assert fn(ptr, prec, a, b, c, st, None, om, None, o, None) == 1, (a, b, c, st, om)
    sim.close()
    gpu.close()


@pytest.mark.parametrize("precision", ["fp32", "fp16s"])
def test_noalloc_observables_all_fluid_without_cell_types(precision):
    """A periodic lattice: no cell-type array (NULL = every cell fluid)."""
    torch = pytest.importorskip("torch")
    import strouhal_gb300 as sg

    fn = _entry(sg)
    gpu = sg.GPU(0)
    nx, ny, nz = 32, 24, 20
    omega = 1.9
    sim = sg.Simulation(gpu, precision=precision, nx=nx, ny=ny, nz=nz, omega=omega)
    sim.initField(2, 0.05)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    prec = 0 if precision == "fp32" else 1
    for call in range(2):
        sim.run(4)
        state = torch.from_numpy(sim.downloadState()).cuda()
        rc = fn(state.data_ptr(), prec, nx, ny, nz, nx * ny * nz, None, omega, None,
                out.data_ptr(), None)
        assert rc == 0, sg.lib().stro_last_error()
        torch.cuda.synchronize()
        ke, diss = out.cpu().numpy()
        assert np.isclose(ke, sim.kineticEnergySum(), rtol=1e-12, atol=0), (call, ke)
        assert np.isclose(diss, sim.dissipationSum(), rtol=1e-12, atol=0), (call, diss)
    sim.close()
    gpu.close()
