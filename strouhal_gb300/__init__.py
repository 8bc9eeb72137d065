"""strouhal_gb300 — GB300-native D3Q19 lattice-Boltzmann step behind a C ABI.

Python mirror (ctypes) of the reference's StrouhalCore solver API
(Sources/StrouhalCore/Sim.swift): `GPU`, `Simulation`, `Precision`, `Cell`,
`StrouhalError` and `trtOmegas`, plus the solid-fraction generators of
CaseSetups.swift. Every call goes through libstrouhal_gb300.so
(include/strouhal_c.h); there is no CPU fallback — importing the wrapper
without the built library, or running without a CUDA device, raises.
"""
import ctypes
import enum
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libstrouhal_gb300.so")

_lib = None
_P = ctypes.c_void_p


class StrouhalError(RuntimeError):
    """Mirror of StrouhalError (Sim.swift:127-136); `code` is the C status."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class Precision(str, enum.Enum):
    """Sim.swift:5-8. fp32 storage or Lehmann-shifted fp16 storage (FP32 math)."""
    fp32 = "fp32"
    fp16s = "fp16s"

    @property
    def ddfBytes(self):
        return 4 if self is Precision.fp32 else 2


# Arithmetic of the step, indexed by STRO_ARITH_* (see Simulation.arithmetic).
ARITHMETICS = ("reference", "fused")
OUTFLOW_MODES = ("dormant", "pressure")
COLLISIONS = ("reference", "kbc")


class Cell(enum.IntEnum):
    """Sim.swift:46-52."""
    fluid = 0
    solid = 1
    lid = 2
    inflow = 3
    outflow = 4


class _Desc(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("nz", ctypes.c_int32), ("omega", ctypes.c_float), ("omega_minus", ctypes.c_float),
                ("lid", ctypes.c_float * 3), ("uin", ctypes.c_float),
                ("ramp_steps", ctypes.c_int32), ("force", ctypes.c_float * 3),
                ("c_smago", ctypes.c_float), ("wants_forces", ctypes.c_int32)]


class StatUQ(ctypes.Structure):
    """stro_stat_uq"""
    _fields_ = [("mean", ctypes.c_double), ("half_width95", ctypes.c_double),
                ("lag1", ctypes.c_double), ("batches", ctypes.c_int32),
                ("trustworthy", ctypes.c_int32)]


class LadderRungC(ctypes.Structure):
    """stro_ladder_rung"""
    _fields_ = [("cells_per_feature", ctypes.c_int32), ("value", ctypes.c_double),
                ("stat", ctypes.c_double)]


class NumUQ(ctypes.Structure):
    """stro_num_uq"""
    _fields_ = [("u_num", ctypes.c_double), ("observed_order", ctypes.c_double),
                ("has_order", ctypes.c_int32), ("note", ctypes.c_int32)]


class DomainVerdict(ctypes.Structure):
    """stro_domain_verdict"""
    _fields_ = [("verdict", ctypes.c_int32), ("anchor", ctypes.c_int32),
                ("distance", ctypes.c_double), ("factor", ctypes.c_double),
                ("reasons", ctypes.c_int32)]


def lib():
    """Load the C-ABI library (built by __graft_entry__.build() / build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise StrouhalError(-1, "libstrouhal_gb300.so is not built (%s); run "
                                "python -c 'import __graft_entry__ as g; g.build()'" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    c_int, c_float, c_double, c_i64 = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_int64
    sig = {
        "stro_last_error": ([], ctypes.c_char_p),
        "stro_abi_version": ([], c_int),
        "stro_ctx_create": ([c_int, ctypes.POINTER(_P)], c_int),
        "stro_ctx_destroy": ([_P], c_int),
        "stro_ctx_info": ([_P, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(c_int)], c_int),
        "stro_sim_create": ([_P, ctypes.POINTER(_Desc), _P, ctypes.POINTER(_P)], c_int),
        "stro_sim_destroy": ([_P], c_int),
        "stro_sim_set_omega": ([_P, c_float, c_float], c_int),
        "stro_sim_set_lid": ([_P, _P], c_int),
        "stro_sim_set_uin": ([_P, c_float], c_int),
        "stro_sim_set_ramp_steps": ([_P, ctypes.c_int32], c_int),
        "stro_sim_set_force": ([_P, _P], c_int),
        "stro_sim_set_c_smago": ([_P, c_float], c_int),
        "stro_sim_set_inflow_uniform": ([_P, c_int], c_int),
        "stro_sim_set_sponge": ([_P, c_int, c_float, c_float, c_float], c_int),
        "stro_sim_set_solid_fractions": ([_P, _P], c_int),
        "stro_sim_set_force_field": ([_P, _P], c_int),
        "stro_sim_init_field": ([_P, ctypes.c_uint32, c_float], c_int),
        "stro_sim_upload_state": ([_P, _P, ctypes.c_size_t], c_int),
        "stro_sim_download_state": ([_P, _P, ctypes.c_size_t], c_int),
        "stro_sim_state_bytes": ([_P, ctypes.POINTER(ctypes.c_size_t)], c_int),
        "stro_sim_run": ([_P, c_i64], c_int),
        "stro_sim_steps_done": ([_P, ctypes.POINTER(c_i64)], c_int),
        "stro_sim_set_steps_done": ([_P, c_i64], c_int),
        "stro_sim_gpu_seconds": ([_P, ctypes.POINTER(c_double)], c_int),
        "stro_sim_moments": ([_P, _P], c_int),
        "stro_sim_probe_force": ([_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, _P], c_int),
        "stro_sim_kinetic_energy": ([_P, ctypes.POINTER(c_double)], c_int),
        "stro_sim_dissipation": ([_P, ctypes.POINTER(c_double)], c_int),
        "stro_sim_observables": ([_P, _P], c_int),
        "stro_sim_digest": ([_P, ctypes.c_char_p], c_int),
        "stro_sim_mass": ([_P, ctypes.POINTER(c_double)], c_int),
        "stro_sim_check_finite": ([_P, ctypes.POINTER(c_int)], c_int),
        "stro_sim_set_variant": ([_P, ctypes.c_int32], c_int),
        "stro_sim_set_rows_tile": ([_P, ctypes.c_int32, ctypes.c_int32], c_int),
        "stro_sim_set_spin_limit": ([_P, ctypes.c_int64], c_int),
        "stro_sim_set_arithmetic": ([_P, ctypes.c_int32], c_int),
        "stro_sim_set_outflow_mode": ([_P, ctypes.c_int32], c_int),
        "stro_sim_set_collision": ([_P, ctypes.c_int32], c_int),
        "stro_sim_get_collision": ([_P, ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_get_outflow_mode": ([_P, ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_render_slice": ([_P, ctypes.c_int32, c_float, _P, ctypes.POINTER(c_double)], c_int),
        "stro_sim_set_pair_block": ([_P, ctypes.c_int32, ctypes.c_int32], c_int),
        "stro_sim_get_pair_block": ([_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_last_path": ([_P, ctypes.c_char_p, ctypes.c_size_t], c_int),
        "stro_sim_split_blocks": ([_P, _P, _P, _P], c_int),
        "stro_sim_get_arithmetic": ([_P, ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_get_rows_tile": ([_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_set_block_split": ([_P, ctypes.c_int32], c_int),
        "stro_sim_set_graphs": ([_P, ctypes.c_int32], c_int),
        "stro_sim_get_variant": ([_P, ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_set_block": ([_P, ctypes.c_int32, ctypes.c_int32], c_int),
        "stro_sim_get_block": ([_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)], c_int),
        "stro_sim_autotune": ([_P, c_i64, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                               ctypes.POINTER(c_double)], c_int),
        "stro_batch_create": ([_P, ctypes.c_int32, _P, ctypes.POINTER(_P)], c_int),
        "stro_batch_destroy": ([_P], c_int),
        "stro_batch_set_mode": ([_P, ctypes.c_int32], c_int),
        "stro_batch_set_tile": ([_P, ctypes.c_int32, ctypes.c_int32], c_int),
        "stro_batch_set_spin_limit": ([_P, c_i64], c_int),
        "stro_batch_set_split": ([_P, ctypes.c_int32], c_int),
        "stro_batch_split_tiles": ([_P, _P, _P], c_int),
        "stro_batch_run": ([_P, _P, _P, _P, ctypes.c_int32, _P], c_int),
        "stro_batch_gpu_seconds": ([_P, ctypes.POINTER(c_double)], c_int),
        "stro_batch_run_sampled": ([_P, _P, _P, _P, _P, _P, _P, _P], c_int),
        "stro_batch_last_path": ([_P, ctypes.c_char_p, ctypes.c_size_t], c_int),
        "stro_batch_autotune": ([_P, c_i64, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                                 ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(c_double)], c_int),
        "stro_adj_create": ([_P, _P, _P, c_i64, ctypes.c_int32, ctypes.POINTER(_P)], c_int),
        "stro_adj_destroy": ([_P], c_int),
        "stro_adj_forward": ([_P, ctypes.POINTER(c_double)], c_int),
        "stro_adj_backward": ([_P, _P, _P], c_int),
        "stro_adj_set_dissipation": ([_P, ctypes.c_int64], c_int),
        "stro_adj_stats": ([_P, ctypes.POINTER(c_double), ctypes.POINTER(c_double),
                            ctypes.POINTER(c_double), ctypes.POINTER(c_i64)], c_int),
        "stro_sha256_hex": ([_P, ctypes.c_size_t, ctypes.c_char_p], c_int),
        "stro_host_alloc": ([ctypes.c_size_t, ctypes.POINTER(_P)], c_int),
        "stro_host_free": ([_P], c_int),
        "stro_disk_solid_fractions": ([ctypes.c_int32, ctypes.c_int32, c_double, c_double,
                                       c_double, _P], c_int),
        "stro_stl_triangle_count": ([_P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32)], c_int),
        "stro_stl_parse": ([_P, ctypes.c_size_t, _P, _P], c_int),
        "stro_sphere_stl": ([c_float, ctypes.c_int32, ctypes.c_int32, _P, ctypes.c_size_t,
                             ctypes.POINTER(ctypes.c_size_t)], c_int),
        "stro_mesh_solid_fractions": ([_P, _P, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_int32, c_float, _P, _P,
                                       ctypes.POINTER(c_double)], c_int),
        "stro_sim_run_sampled": ([_P, c_i64, c_i64, c_i64, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int32, ctypes.c_int32, _P, c_i64,
                                  ctypes.POINTER(c_i64), _P], c_int),
        "stro_uq_stat": ([_P, c_i64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(StatUQ)], c_int),
        "stro_uq_num": ([_P, ctypes.c_int32, ctypes.POINTER(NumUQ)], c_int),
        "stro_uq_mach": ([c_double, c_double, ctypes.POINTER(c_double)], c_int),
        "stro_uq_classify": ([c_double, c_double, ctypes.c_int32, ctypes.c_char_p,
                              ctypes.POINTER(DomainVerdict)], c_int),
        "stro_uq_anchor": ([ctypes.c_int32, ctypes.c_char_p, ctypes.c_size_t, _P, _P,
                            ctypes.c_char_p, ctypes.c_size_t], c_int),
        "stro_uq_combined": ([c_double, c_double, c_double, ctypes.POINTER(DomainVerdict),
                              ctypes.POINTER(c_double)], c_int),
        "stro_sphere_solid_fractions": ([ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                         c_double, c_double, c_double, c_double, ctypes.c_int32,
                                         _P], c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        msg = lib().stro_last_error().decode("utf-8", "replace")
        raise StrouhalError(rc, msg)


def _f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def trtOmegas(tau, lam=None):
    """tau -> (omega+, omega-) via the TRT magic parameter Lambda (Sim.swift:188-193)."""
    wp = 1.0 / tau
    if lam is None:
        w = float(np.float32(wp))
        return w, w
    tm = 0.5 + lam / (tau - 0.5)
    return float(np.float32(wp)), float(np.float32(1.0 / tm))


class GPU:
    """One CUDA device and one stream (Sim.swift:60-78)."""

    def __init__(self, device=0):
        self._h = _P()
        self.device = int(device)
        _check(lib().stro_ctx_create(int(device), ctypes.byref(self._h)))
        name = ctypes.create_string_buffer(256)
        sms = ctypes.c_int()
        _check(lib().stro_ctx_info(self._h, name, 256, ctypes.byref(sms)))
        self.name = name.value.decode()
        self.smCount = sms.value

    def close(self):
        if self._h:
            lib().stro_ctx_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _flags_array(flags, nx, ny, nz):
    N = nx * ny * nz
    if flags is None:
        return None
    if callable(flags):
        arr = np.zeros((nz, ny, nx), np.uint8)
        for z in range(nz):
            for y in range(ny):
                for x in range(nx):
                    arr[z, y, x] = int(flags(x, y, z))
        return arr.reshape(-1)
    arr = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
    if arr.size != N:
        raise ValueError("flags must hold nx*ny*nz cell codes")
    return arr


class Simulation:
    """Mirror of Simulation (Sim.swift:153-459) over the C ABI.

    `flags` is an array of N cell codes in x-fastest order, or a callable
    flags(x, y, z) -> Cell like the Swift initializer's closure.
    """

    def __init__(self, gpu, precision=Precision.fp32, nx=1, ny=1, nz=1, omega=1.0,
                 omegaMinus=None, lid=(0.0, 0.0, 0.0), uin=0.0, rampSteps=0,
                 force=(0.0, 0.0, 0.0), cSmago=0.0, wantsForces=False, flags=None,
                 arithmetic="reference"):
        self.gpu = gpu
        self.precision = Precision(precision)
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        d = _Desc()
        d.precision = 0 if self.precision is Precision.fp32 else 1
        d.nx, d.ny, d.nz = self.nx, self.ny, self.nz
        d.omega = omega
        d.omega_minus = omega if omegaMinus is None else omegaMinus
        d.lid = _f3(lid)
        d.uin = uin
        d.ramp_steps = int(rampSteps)
        d.force = _f3(force)
        d.c_smago = cSmago
        d.wants_forces = 1 if wantsForces else 0
        fl = _flags_array(flags, self.nx, self.ny, self.nz)
        self._flags = fl
        self._h = _P()
        _check(lib().stro_sim_create(gpu._h, ctypes.byref(d),
                                     None if fl is None else fl.ctypes.data, ctypes.byref(self._h)))
        self._omega = float(np.float32(d.omega))
        self._omegaMinus = float(np.float32(d.omega_minus))
        self._lid = tuple(float(np.float32(v)) for v in lid)
        self._uin = float(np.float32(uin))
        self._ramp = int(rampSteps)
        self._force = tuple(float(np.float32(v)) for v in force)
        self._cSmago = float(np.float32(cSmago))
        self._inflowUniform = False
        self._sponge = None
        if arithmetic != "reference":
            self.arithmetic = arithmetic

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().stro_sim_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self):
        return self.nx * self.ny * self.nz

    # -- mutable properties (Sim.swift:164-172) ----------------------------
    @property
    def omega(self):
        return self._omega

    @omega.setter
    def omega(self, v):
        self._omega = float(np.float32(v))
        _check(lib().stro_sim_set_omega(self._h, self._omega, self._omegaMinus))

    @property
    def omegaMinus(self):
        return self._omegaMinus

    @omegaMinus.setter
    def omegaMinus(self, v):
        self._omegaMinus = float(np.float32(v))
        _check(lib().stro_sim_set_omega(self._h, self._omega, self._omegaMinus))

    @property
    def lidVel(self):
        return self._lid

    @lidVel.setter
    def lidVel(self, v):
        self._lid = tuple(float(np.float32(x)) for x in v)
        _check(lib().stro_sim_set_lid(self._h, _f3(self._lid)))

    @property
    def uinTarget(self):
        return self._uin

    @uinTarget.setter
    def uinTarget(self, v):
        self._uin = float(np.float32(v))
        _check(lib().stro_sim_set_uin(self._h, self._uin))

    @property
    def rampSteps(self):
        return self._ramp

    @rampSteps.setter
    def rampSteps(self, v):
        self._ramp = int(v)
        _check(lib().stro_sim_set_ramp_steps(self._h, self._ramp))

    @property
    def force(self):
        return self._force

    @force.setter
    def force(self, v):
        self._force = tuple(float(np.float32(x)) for x in v)
        _check(lib().stro_sim_set_force(self._h, _f3(self._force)))

    @property
    def cSmago(self):
        return self._cSmago

    @cSmago.setter
    def cSmago(self, v):
        self._cSmago = float(np.float32(v))
        _check(lib().stro_sim_set_c_smago(self._h, self._cSmago))

    @property
    def inflowUniform(self):
        return self._inflowUniform

    @inflowUniform.setter
    def inflowUniform(self, v):
        self._inflowUniform = bool(v)
        _check(lib().stro_sim_set_inflow_uniform(self._h, int(self._inflowUniform)))

    @property
    def sponge(self):
        return self._sponge

    @sponge.setter
    def sponge(self, v):
        """(x0, width, tau) or None."""
        if v is None:
            _check(lib().stro_sim_set_sponge(self._h, 0, 0.0, 0.0, 0.0))
        else:
            _check(lib().stro_sim_set_sponge(self._h, 1, float(v[0]), float(v[1]), float(v[2])))
        self._sponge = v

    # -- set-up ---------------------------------------------------------------
    def setSolidFractions(self, eps):
        eps = np.ascontiguousarray(eps, dtype=np.float32).reshape(-1)
        if eps.size != self.cells:
            raise ValueError("eps must hold one value per cell")
        _check(lib().stro_sim_set_solid_fractions(self._h, eps.ctypes.data))

    def setForceField(self, field):
        """Per-cell Guo force field, shape (3, N) float32 (extension); None removes it."""
        if field is None:
            _check(lib().stro_sim_set_force_field(self._h, None))
            return
        field = np.ascontiguousarray(field, dtype=np.float32).reshape(3, self.cells)
        _check(lib().stro_sim_set_force_field(self._h, field.ctypes.data))

    def initField(self, mode, amplitude):
        _check(lib().stro_sim_init_field(self._h, int(mode), float(amplitude)))

    def _dtype(self):
        return np.float32 if self.precision is Precision.fp32 else np.float16

    def uploadState(self, f):
        f = np.ascontiguousarray(f, dtype=self._dtype())
        if f.size != 19 * self.cells:
            raise ValueError("state must hold 19*N values")
        _check(lib().stro_sim_upload_state(self._h, f.ctypes.data, f.nbytes))

    def downloadState(self, out=None):
        if out is None:
            out = np.empty((19, self.cells), self._dtype())
        _check(lib().stro_sim_download_state(self._h, out.ctypes.data, out.nbytes))
        return out

    # -- stepping ---------------------------------------------------------------
    def run(self, steps):
        _check(lib().stro_sim_run(self._h, int(steps)))

    @property
    def stepsDone(self):
        v = ctypes.c_int64()
        _check(lib().stro_sim_steps_done(self._h, ctypes.byref(v)))
        return v.value

    @stepsDone.setter
    def stepsDone(self, v):
        _check(lib().stro_sim_set_steps_done(self._h, int(v)))

    @property
    def gpuSeconds(self):
        v = ctypes.c_double()
        _check(lib().stro_sim_gpu_seconds(self._h, ctypes.byref(v)))
        return v.value

    # -- probes -----------------------------------------------------------------
    def probeMoments(self):
        out = np.empty((self.cells, 4), np.float32)
        _check(lib().stro_sim_moments(self._h, out.ctypes.data))
        return out

    def probeForce(self, xRange, yRange):
        out = np.zeros(3, np.float64)
        _check(lib().stro_sim_probe_force(self._h, int(xRange[0]), int(xRange[1]),
                                          int(yRange[0]), int(yRange[1]), out.ctypes.data))
        return out

    def runSampled(self, transientSteps, sampleSteps, stride, xRange, yRange):
        """Ladder.measure's stepping (Ladder.swift:54-66) in one submission: the
        transient, then chunk + two-step force probe pairs until sampleSteps
        steps are taken. Returns (forces (n, 3) float64, step count after each
        probe (n,) int64); the samples are read back once."""
        chunk = max(2, int(stride) - 2) & ~1
        n = (int(sampleSteps) + chunk + 1) // (chunk + 2) if sampleSteps > 0 else 0
        forces = np.zeros((max(n, 1), 3), np.float64)
        at = np.zeros(max(n, 1), np.int64)
        got = ctypes.c_int64()
        _check(lib().stro_sim_run_sampled(self._h, int(transientSteps), int(sampleSteps),
                                          int(stride), int(xRange[0]), int(xRange[1]),
                                          int(yRange[0]), int(yRange[1]), forces.ctypes.data,
                                          forces.shape[0], ctypes.byref(got), at.ctypes.data))
        return forces[:got.value], at[:got.value]

    def kineticEnergySum(self):
        v = ctypes.c_double()
        _check(lib().stro_sim_kinetic_energy(self._h, ctypes.byref(v)))
        return v.value

    def dissipationSum(self):
        v = ctypes.c_double()
        _check(lib().stro_sim_dissipation(self._h, ctypes.byref(v)))
        return v.value

    def observables(self):
        """(kineticEnergySum(), dissipationSum()) from one reduction."""
        out = (ctypes.c_double * 2)()
        _check(lib().stro_sim_observables(self._h, out))
        return out[0], out[1]

    @property
    def stateDigest(self):
        buf = ctypes.create_string_buffer(65)
        _check(lib().stro_sim_digest(self._h, buf))
        return buf.value.decode()

    def massSum(self):
        v = ctypes.c_double()
        _check(lib().stro_sim_mass(self._h, ctypes.byref(v)))
        return v.value

    def renderSlice(self, z, uref, timing=False):
        """The |u| colormap of slice z (Kernels.metal:465-500) as an (ny, nx, 4)
        float16 RGBA image, rows as the reference's texture write (y flipped)."""
        out = np.zeros((self.ny, self.nx, 4), np.float16)
        sec = ctypes.c_double()
        _check(lib().stro_sim_render_slice(self._h, int(z), float(uref), out.ctypes.data,
                                           ctypes.byref(sec)))
        return (out, sec.value) if timing else out

    def checkFinite(self):
        v = ctypes.c_int()
        _check(lib().stro_sim_check_finite(self._h, ctypes.byref(v)))
        return bool(v.value)

    # -- launch shape ---------------------------------------------------------
    @property
    def block(self):
        bx, by = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().stro_sim_get_block(self._h, ctypes.byref(bx), ctypes.byref(by)))
        return bx.value, by.value

    @block.setter
    def block(self, v):
        _check(lib().stro_sim_set_block(self._h, int(v[0]), int(v[1])))

    @property
    def variant(self):
        v = ctypes.c_int32()
        _check(lib().stro_sim_get_variant(self._h, ctypes.byref(v)))
        return v.value

    @variant.setter
    def variant(self, v):
        _check(lib().stro_sim_set_variant(self._h, int(v)))

    @property
    def arithmetic(self):
        """'reference' (the reference's expressions as written) or 'fused'
        (fused multiply-adds, fewer instructions; stro_sim_set_arithmetic)."""
        v = ctypes.c_int32()
        _check(lib().stro_sim_get_arithmetic(self._h, ctypes.byref(v)))
        return ARITHMETICS[v.value]

    @arithmetic.setter
    def arithmetic(self, v):
        if v not in ARITHMETICS:
            raise ValueError("arithmetic must be one of %s" % (ARITHMETICS,))
        _check(lib().stro_sim_set_arithmetic(self._h, ARITHMETICS.index(v)))

    @property
    def collision(self):
        """'reference' (the reference's SRT / TRT) or 'kbc' (the KBC entropic
        collision; stro_sim_set_collision)."""
        v = ctypes.c_int32()
        _check(lib().stro_sim_get_collision(self._h, ctypes.byref(v)))
        return COLLISIONS[v.value]

    @collision.setter
    def collision(self, v):
        if v not in COLLISIONS:
            raise ValueError("collision must be one of %s" % (COLLISIONS,))
        _check(lib().stro_sim_set_collision(self._h, COLLISIONS.index(v)))

    @property
    def outflowMode(self):
        """Outflow walls: 'dormant' (the reference's sign-flip reflection) or
        'pressure' (anti-bounce-back at rho = 1 with its velocity terms;
        stro_sim_set_outflow_mode)."""
        v = ctypes.c_int32()
        _check(lib().stro_sim_get_outflow_mode(self._h, ctypes.byref(v)))
        return OUTFLOW_MODES[v.value]

    @outflowMode.setter
    def outflowMode(self, v):
        if v not in OUTFLOW_MODES:
            raise ValueError("outflowMode must be one of %s" % (OUTFLOW_MODES,))
        _check(lib().stro_sim_set_outflow_mode(self._h, OUTFLOW_MODES.index(v)))

    @property
    def pairBlock(self):
        """(bx, 1): launch shape of the FP16 pair variant 1."""
        bx, by = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().stro_sim_get_pair_block(self._h, ctypes.byref(bx), ctypes.byref(by)))
        return bx.value, by.value

    @pairBlock.setter
    def pairBlock(self, v):
        _check(lib().stro_sim_set_pair_block(self._h, int(v[0]), int(v[1])))

    @property
    def lastPath(self):
        """Kernel path of the latest step launch (stro_sim_last_path)."""
        buf = ctypes.create_string_buffer(32)
        _check(lib().stro_sim_last_path(self._h, buf, 32))
        return buf.value.decode()

    @property
    def splitBlocks(self):
        """(bulk, x-face, boundary) block counts of the split's last lists."""
        bu, fa, ed = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(lib().stro_sim_split_blocks(self._h, ctypes.byref(bu), ctypes.byref(fa),
                                           ctypes.byref(ed)))
        return bu.value, fa.value, ed.value

    @property
    def rowsTile(self):
        """(threads per block, lattice rows per tile) of the row-staged variant 2."""
        t, r = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().stro_sim_get_rows_tile(self._h, ctypes.byref(t), ctypes.byref(r)))
        return t.value, r.value

    @rowsTile.setter
    def rowsTile(self, v):
        _check(lib().stro_sim_set_rows_tile(self._h, int(v[0]), int(v[1])))

    def setSpinLimit(self, polls):
        """Polls per bounded wait of the row-staged variant (0: give up at once)."""
        _check(lib().stro_sim_set_spin_limit(self._h, int(polls)))

    def setBlockSplit(self, enabled):
        """Bulk blocks of a walled lattice on the wall-free kernels and blocks at
        velocity-inflow x faces on the x-face kernels (default True); "columns"
        also orders the boundary blocks' odd pass column by column; "noface"
        runs the x-face blocks on the wall-aware kernels; "merged" runs the bulk
        and x-face blocks in one launch; "pair" does that with the bulk blocks
        of an FP16-storage lattice two cells per thread."""
        modes = {"columns": 2, "noface": 3, "merged": 4, "pair": 5}
        mode = modes.get(enabled) if isinstance(enabled, str) else int(bool(enabled))
        if mode is None:
            raise ValueError("block split: True, False, 'columns', 'noface', 'merged' or 'pair'")
        _check(lib().stro_sim_set_block_split(self._h, mode))

    def setGraphs(self, enabled):
        """Replay CUDA graphs of plain steps past the ramp (default True)."""
        _check(lib().stro_sim_set_graphs(self._h, int(bool(enabled))))

    def autotune(self, steps=20):
        """Pick the fastest kernel variant and launch shape (state restored); returns (bx, by, GLUPS)."""
        bx, by, g = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        _check(lib().stro_sim_autotune(self._h, int(steps), ctypes.byref(bx), ctypes.byref(by),
                                       ctypes.byref(g)))
        return bx.value, by.value, g.value


class Batch:
    """Several simulations of one precision advanced together (stro_batch_*).

    mode: "persistent" (one cooperative kernel in a CUDA graph), "rounds" (a
    graph of one launch per round), "sequential" (one instance after another,
    the reference's order) or "streams" (every instance on its own stream with
    its own kernels and step graphs, all enqueued at once)."""

    MODES = {"persistent": 0, "rounds": 1, "sequential": 2, "streams": 3}

    def __init__(self, gpu, sims, mode="persistent"):
        self.sims = list(sims)
        arr = (_P * len(self.sims))(*[s._h for s in self.sims])
        self._h = _P()
        _check(lib().stro_batch_create(gpu._h, len(self.sims), arr, ctypes.byref(self._h)))
        self.mode = mode

    @property
    def mode(self):
        return self._mode

    @mode.setter
    def mode(self, m):
        _check(lib().stro_batch_set_mode(self._h, self.MODES[m]))
        self._mode = m

    def setTile(self, bx, by):
        _check(lib().stro_batch_set_tile(self._h, int(bx), int(by)))

    def setSpinLimit(self, polls):
        _check(lib().stro_batch_set_spin_limit(self._h, int(polls)))

    def setSplit(self, on):
        """Rounds mode on walled lattices: bulk tiles on the wall-free kernels."""
        _check(lib().stro_batch_set_split(self._h, 1 if on else 0))

    @property
    def splitTiles(self):
        """(bulk, boundary) tiles of the last run; (0, 0) when it ran unsplit."""
        bu, ed = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().stro_batch_split_tiles(self._h, ctypes.byref(bu), ctypes.byref(ed)))
        return bu.value, ed.value

    def run(self, steps, logEvery=None):
        """Advance sims[i] by steps[i]; returns kinetic-energy traces (lists) or None."""
        n = len(self.sims)
        st = np.ascontiguousarray(steps, dtype=np.int64).reshape(n)
        if logEvery is None:
            _check(lib().stro_batch_run(self._h, st.ctypes.data, None, None, 0, None))
            return None
        le = np.ascontiguousarray(logEvery, dtype=np.int32).reshape(n)
        stride = int(max(1, max((s // l + 1) if l > 0 else 0 for s, l in zip(st, le))))
        tr = np.zeros((n, stride), np.float64)
        cnt = np.zeros(n, np.int32)
        _check(lib().stro_batch_run(self._h, st.ctypes.data, le.ctypes.data, tr.ctypes.data,
                                    stride, cnt.ctypes.data))
        return [tr[i, :cnt[i]].copy() for i in range(n)]

    def runSampled(self, transientSteps, sampleSteps, strides, boxes):
        """Simulation.runSampled for every member in one submission; boxes[i] =
        (xRange, yRange). Returns a list of (forces (n_i, 3), step counts (n_i,))."""
        n = len(self.sims)
        tr = np.ascontiguousarray(transientSteps, np.int64).reshape(n)
        sa = np.ascontiguousarray(sampleSteps, np.int64).reshape(n)
        sd = np.ascontiguousarray(strides, np.int64).reshape(n)
        bx = np.ascontiguousarray([[b[0][0], b[0][1], b[1][0], b[1][1]] for b in boxes],
                                  np.int32).reshape(n, 4)
        t0 = [s.stepsDone for s in self.sims]
        chunks = [max(2, int(s) - 2) & ~1 for s in sd]
        counts = [(int(a) + c + 1) // (c + 2) if a > 0 else 0 for a, c in zip(sa, chunks)]
        bufs = [np.zeros((max(c, 1), 3), np.float64) for c in counts]
        ptrs = (_P * n)(*[b.ctypes.data for b in bufs])
        cap = np.ascontiguousarray([b.shape[0] for b in bufs], np.int64)
        got = np.zeros(n, np.int64)
        _check(lib().stro_batch_run_sampled(self._h, tr.ctypes.data, sa.ctypes.data, sd.ctypes.data,
                                            bx.ctypes.data, ptrs, cap.ctypes.data,
                                            got.ctypes.data))
        out = []
        for i in range(n):
            k = int(got[i])
            T = int(tr[i]) & ~1
            at = t0[i] + T + (np.arange(1, k + 1, dtype=np.int64) * (chunks[i] + 2))
            out.append((bufs[i][:k], at))
        return out

    @property
    def gpuSeconds(self):
        v = ctypes.c_double()
        _check(lib().stro_batch_gpu_seconds(self._h, ctypes.byref(v)))
        return v.value

    @property
    def lastPath(self):
        buf = ctypes.create_string_buffer(64)
        _check(lib().stro_batch_last_path(self._h, buf, 64))
        return buf.value.decode()

    def autotune(self, rounds=20):
        m, bx, by, sec = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
        _check(lib().stro_batch_autotune(self._h, int(rounds), ctypes.byref(m), ctypes.byref(bx),
                                         ctypes.byref(by), ctypes.byref(sec)))
        self._mode = {v: k for k, v in self.MODES.items()}[m.value]
        return self._mode, bx.value, by.value, sec.value

    def close(self):
        if getattr(self, "_h", None):
            lib().stro_batch_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Adjoint:
    """Discrete adjoint of a time-averaged objective over a window (stro_adj_*).

    Default objective: J = mean over the odd steps of direction . F_box, F_box
    the force the probe box sums. With dissipationEvery = m (even): J = mean
    of the dissipation sum (dissipationSum) of the states after m, 2m, ...
    steps of the window (box and direction unused). forward() advances the
    simulation through the window and returns J; backward() returns
    (dJ/d eps, dJ/d F_field) as float32 arrays of shapes (N,) and (3, N)."""

    def __init__(self, sim, steps, box=None, direction=(1.0, 0.0, 0.0), checkpoints=8,
                 dissipationEvery=None):
        self.sim = sim
        if box is None:
            if dissipationEvery is None:
                raise ValueError("the force objective needs a probe box")
            box = ((0, 0), (0, 0))  # unused by the dissipation objective
        d3 = (ctypes.c_double * 3)(*[float(v) for v in direction])
        b4 = (ctypes.c_int32 * 4)(int(box[0][0]), int(box[0][1]), int(box[1][0]), int(box[1][1]))
        self._h = _P()
        _check(lib().stro_adj_create(sim._h, d3, b4, int(steps), int(checkpoints),
                                     ctypes.byref(self._h)))
        if dissipationEvery is not None:
            try:
                _check(lib().stro_adj_set_dissipation(self._h, int(dissipationEvery)))
            except Exception:
                self.close()
                raise

    def forward(self):
        J = ctypes.c_double()
        _check(lib().stro_adj_forward(self._h, ctypes.byref(J)))
        return J.value

    def backward(self):
        N = self.sim.cells
        ge = np.zeros(N, np.float32)
        gf = np.zeros((3, N), np.float32)
        _check(lib().stro_adj_backward(self._h, ge.ctypes.data, gf.ctypes.data))
        return ge, gf

    def stats(self):
        f, r, a, k = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
        _check(lib().stro_adj_stats(self._h, ctypes.byref(f), ctypes.byref(r), ctypes.byref(a),
                                    ctypes.byref(k)))
        return {"forward_s": f.value, "recompute_s": r.value, "adjoint_s": a.value,
                "adjoint_steps": k.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().stro_adj_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sha256Hex(data):
    """SHA-256 of a bytes-like object or array, computed by the library."""
    buf = np.ascontiguousarray(np.frombuffer(memoryview(data).cast("B"), np.uint8))
    out = ctypes.create_string_buffer(65)
    _check(lib().stro_sha256_hex(buf.ctypes.data, buf.nbytes, out))
    return out.value.decode()


class PinnedBuffer:
    """Page-locked host array (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, shape, dtype):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self._p = _P()
        _check(lib().stro_host_alloc(self.nbytes, ctypes.byref(self._p)))
        raw = (ctypes.c_uint8 * self.nbytes).from_address(self._p.value)
        self.array = np.frombuffer(raw, np.uint8).view(dtype).reshape(shape)

    def close(self):
        if self._p:
            self.array = None
            lib().stro_host_free(self._p)
            self._p = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def diskSolidFractions(nx, ny, cx, cy, r):
    """CaseSetups.swift:6-25 (16x16 subcells), computed in the C++ runtime."""
    out = np.zeros(nx * ny, np.float32)
    _check(lib().stro_disk_solid_fractions(nx, ny, cx, cy, r, out.ctypes.data))
    return out


def sphereSolidFractions(nx, ny, nz, cx, cy, cz, r, sub=8):
    """CaseSetups.swift:68-90 (sub^3 subcells), computed in the C++ runtime."""
    out = np.zeros(nx * ny * nz, np.float32)
    _check(lib().stro_sphere_solid_fractions(nx, ny, nz, cx, cy, cz, r, sub, out.ctypes.data))
    return out


class StlMesh:
    """Binary-STL triangle soup (StlVoxels.swift:6-43): `triangles` is a
    (count, 3, 3) float32 array of vertices, `boundsMin` / `boundsMax` the
    componentwise bounds."""

    def __init__(self, binarySTL):
        data = bytes(binarySTL)
        buf = ctypes.create_string_buffer(data, len(data))
        n = ctypes.c_uint32()
        _check(lib().stro_stl_triangle_count(buf, len(data), ctypes.byref(n)))
        tris = np.zeros((n.value, 3, 3), np.float32)
        bounds = np.zeros(6, np.float32)
        _check(lib().stro_stl_parse(buf, len(data), tris.ctypes.data, bounds.ctypes.data))
        self.triangles = tris
        self.boundsMin = bounds[:3].copy()
        self.boundsMax = bounds[3:].copy()


def sphereSTLData(radius, segments=48, rings=24):
    """StlVoxels.swift:120-143: a lat-long sphere as binary STL bytes."""
    n = ctypes.c_size_t()
    _check(lib().stro_sphere_stl(radius, segments, rings, None, 0, ctypes.byref(n)))
    out = ctypes.create_string_buffer(n.value)
    _check(lib().stro_sphere_stl(radius, segments, rings, out, n.value, ctypes.byref(n)))
    return out.raw


def meshSolidFractions(gpu, mesh, nx, ny, nz, scale, offset, timing=False):
    """StlVoxels.swift:52-117 on the GPU. `mesh` is an StlMesh or a (count, 3, 3)
    triangle array; returns nx*ny*nz float32 fractions (and the device seconds
    of the ray kernel with timing=True)."""
    tris = np.ascontiguousarray(getattr(mesh, "triangles", mesh), dtype=np.float32).reshape(-1, 9)
    off = np.ascontiguousarray(offset, dtype=np.float32).reshape(3)
    out = np.zeros(int(nx) * int(ny) * int(nz), np.float32)
    sec = ctypes.c_double()
    _check(lib().stro_mesh_solid_fractions(gpu._h, tris.ctypes.data if tris.size else None,
                                           tris.shape[0], nx, ny, nz, scale, off.ctypes.data,
                                           out.ctypes.data, ctypes.byref(sec)))
    return (out, sec.value) if timing else out
