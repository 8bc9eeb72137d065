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
    # sizes beyond what the entry point accepts are refused, not attempted
    rc = fn(state.data_ptr(), prec, 2048, 2048, 1024, 1 << 33, None, omega, None,
            out.data_ptr(), None)
    assert rc == 1
    sim.close()
    gpu.close()
