"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

`OracleSim` drives the scalar restatement in lbm_oracle.cpp with the same
set-up and run semantics as the reference's `Simulation`
(Sources/StrouhalCore/Sim.swift:195-458): per-cell flags, neighbour masks,
per-step uniforms with the cosine ramp, AA parity, the two-step force probe,
moments, mass sum and SHA-256 state digest. With backend="ref" the same driver
runs the reference's own kernel source compiled as C++ (oracle/_ref), which is
how the restatement is pinned.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg; the product never loads anything from oracle/.
"""
import ctypes
import hashlib
import os
import struct

import numpy as np

from . import build_oracle as _build

KIND_F32, KIND_F16, KIND_F64 = 0, 1, 2
_DTYPES = {KIND_F32: np.float32, KIND_F16: np.float16, KIND_F64: np.float64}
# step kinds of the fused-multiply-add arithmetic over FP32 / FP16 storage
_FUSED_STEP_KIND = {KIND_F32: 3, KIND_F16: 4}
ORC_PRESSURE_OUTFLOW = 0x100  # orc_step kind flag: outflow walls with the pressure terms
ORC_KBC = 0x200               # orc_step kind flag: the KBC collision

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])
OPP = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17])

FLUID, SOLID, LID, INFLOW, OUTFLOW = 0, 1, 2, 3, 4

_lib = None
_ref = None
_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.oracle_lib_path()
        src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lbm_oracle.cpp")
        if not os.path.exists(path) or (os.path.exists(src) and
                                        os.path.getmtime(src) > os.path.getmtime(path)):
            _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_masks.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P]
        L.orc_params.argtypes = ([_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.c_longlong, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_longlong, ctypes.c_float, _P,
                                  ctypes.c_int, _P, ctypes.c_int, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_float, ctypes.c_int])
        L.orc_step.argtypes = [ctypes.c_int, _P, _P, _P, _P, _P, _P, _P, _P, ctypes.c_int]
        L.orc_moments.argtypes = [ctypes.c_int, _P, _P, _P, _P, _P]
        L.orc_init_field.argtypes = [ctypes.c_int, _P, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                     ctypes.c_float]
        L.orc_adjoint_force.argtypes = [_P, _P, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P, _P, _P,
                                        _P]
        L.orc_adjoint_force_ex.argtypes = ([ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_int, _P,
                                            _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, _P, _P])
        L.orc_adjoint_dissipation_ex.argtypes = ([ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_double, _P, _P,
                                                  ctypes.c_int, ctypes.c_int, _P, _P, _P])
        L.orc_mass.argtypes = [ctypes.c_int, _P, ctypes.c_size_t]
        L.orc_observables.argtypes = [ctypes.c_int, _P, _P, _P, _P, ctypes.c_double,
                                      ctypes.c_int, _P]
        L.orc_mesh_solid_fractions.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_float, _P, _P]
        L.orc_colorize.argtypes = [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_float, ctypes.c_int, _P]
        L.orc_mass.restype = ctypes.c_double
        _lib = L
    return _lib


def ref_lib():
    """The reference's kernel source compiled as C++, or None when unavailable."""
    global _ref
    if _ref is None:
        path = _build.ref_lib_path()
        if not os.path.exists(path):
            if _build.build_ref() is None:
                return None
        L = ctypes.CDLL(path)
        L.ref_step.argtypes = [ctypes.c_int, _P, _P, _P, _P, _P, _P, _P]
        L.ref_moments.argtypes = [ctypes.c_int, _P, _P, _P, _P]
        L.ref_init_field.argtypes = [ctypes.c_int, _P, _P]
        L.ref_colorize.argtypes = [_P, _P, _P, _P, _P]
        _ref = L
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data


def trt_omegas(tau, lam=None):
    """tau -> (omega+, omega-), Sim.swift:188-193 (lam None = SRT)."""
    wp = 1.0 / tau
    if lam is None:
        return float(np.float32(wp)), float(np.float32(wp))
    tm = 0.5 + lam / (tau - 0.5)
    return float(np.float32(wp)), float(np.float32(1.0 / tm))


def masks(flags, nx, ny, nz):
    flags = np.ascontiguousarray(flags, dtype=np.uint8)
    sm = np.zeros(nx * ny * nz, np.uint32)
    lm = np.zeros(nx * ny * nz, np.uint32)
    lib().orc_masks(_ptr(flags), nx, ny, nz, _ptr(sm), _ptr(lm))
    return sm, lm


def flags_from(fn, nx, ny, nz):
    """Evaluate a flags(x, y, z) -> Cell callable in the reference's x-fastest order."""
    fl = np.zeros(nx * ny * nz, np.uint8)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                fl[(z * ny + y) * nx + x] = int(fn(x, y, z))
    return fl


class OracleSim:
    """CPU mirror of `Simulation` over the oracle (or the compiled reference)."""

    def __init__(self, nx, ny, nz, omega, omegaMinus=None, lid=(0.0, 0.0, 0.0), uin=0.0,
                 rampSteps=0, force=(0.0, 0.0, 0.0), cSmago=0.0, wantsForces=False,
                 flags=None, kind=KIND_F32, backend="oracle", threads=1, arithmetic="reference"):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.N = self.nx * self.ny * self.nz
        self.kind = kind
        if arithmetic not in ("reference", "fused"):
            raise ValueError("arithmetic must be 'reference' or 'fused'")
        if arithmetic == "fused" and (kind not in _FUSED_STEP_KIND or backend != "oracle"):
            raise ValueError("the fused arithmetic exists for FP32 arithmetic in the oracle only")
        self.arithmetic = arithmetic
        self.step_kind = _FUSED_STEP_KIND[kind] if arithmetic == "fused" else kind
        self.backend = backend
        self.threads = threads
        if backend == "ref" and kind == KIND_F64:
            raise ValueError("the reference source has no FP64 build")
        self.omega = float(np.float32(omega))
        self.omegaMinus = float(np.float32(omega if omegaMinus is None else omegaMinus))
        self.lidVel = tuple(float(np.float32(v)) for v in lid)
        self.uinTarget = float(np.float32(uin))
        self.rampSteps = int(rampSteps)
        self.force = tuple(float(np.float32(v)) for v in force)
        self.cSmago = float(np.float32(cSmago))
        self.inflowUniform = False
        self.sponge = None
        # outflow walls: "dormant" (the reference's sign flip) or "pressure"
        # (anti-bounce-back with its velocity terms, the library's extension)
        self.outflowMode = "dormant"
        # "reference" (SRT / TRT) or "kbc" (the library's KBC collision)
        self.collision = "reference"
        self.stepsDone = 0
        self.f = np.zeros((19, self.N), _DTYPES[kind])
        if flags is None:
            self.flags = np.zeros(self.N, np.uint8)
        elif callable(flags):
            self.flags = flags_from(flags, self.nx, self.ny, self.nz)
        else:
            self.flags = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1).copy()
        self.solidMask, self.lidMask = masks(self.flags, self.nx, self.ny, self.nz)
        fdt = np.float64 if kind == KIND_F64 else np.float32
        self.forceBuf = np.zeros((self.N, 4), fdt) if wantsForces else None
        self.eps = None
        self.forceField = None
        self._force_steps = set()

    # -- set-up -------------------------------------------------------------
    def setSolidFractions(self, eps):
        eps = np.ascontiguousarray(eps, dtype=np.float32).reshape(-1)
        assert eps.size == self.N
        self.eps = eps.copy()

    def setForceField(self, field):
        """Per-cell Guo force field, shape (3, N) float32; None clears it."""
        if field is None:
            self.forceField = None
            return
        field = np.ascontiguousarray(field, dtype=np.float32).reshape(3, self.N)
        if self.backend == "ref":
            raise ValueError("the reference has no per-cell force field")
        self.forceField = field.copy()

    def initField(self, mode, amplitude):
        tau = float(np.float32(1.0) / np.float32(self.omega))
        if self.backend == "ref":
            ip = struct.pack("4I4f", self.nx, self.ny, self.nz, mode, amplitude, tau, 0.0, 0.0)
            ref_lib().ref_init_field(int(self.kind == KIND_F16), _ptr(self.f), ip)
        else:
            lib().orc_init_field(self.kind, _ptr(self.f), self.nx, self.ny, self.nz, mode,
                                 amplitude, tau)

    # -- stepping -----------------------------------------------------------
    def params(self, step, writeForce=False):
        buf = ctypes.create_string_buffer(80)
        f3 = (ctypes.c_float * 3)(*self.force)
        l3 = (ctypes.c_float * 3)(*self.lidVel)
        if self.sponge is None:
            sx0, sw, stau = 1e9, 0.0, 1.0
        else:
            sx0, sw, stau = self.sponge
        lib().orc_params(buf, self.nx, self.ny, self.nz, step, self.omega, self.omegaMinus,
                         self.uinTarget, self.rampSteps, self.cSmago, f3, int(writeForce), l3,
                         int(self.inflowUniform), sx0, sw, stau, int(self.eps is not None))
        return buf.raw

    def run(self, steps):
        dummy_eps = np.zeros(4, np.float32)
        for _ in range(int(steps)):
            t = self.stepsDone
            p = self.params(t, writeForce=(t in self._force_steps))
            eps = self.eps if self.eps is not None else dummy_eps
            if self.backend == "ref":
                if self.outflowMode != "dormant" or self.collision != "reference":
                    raise ValueError("the reference source has the dormant outflow wall and "
                                     "the SRT / TRT collision only")
                force = self.forceBuf if self.forceBuf is not None else np.zeros((1, 4), np.float32)
                ref_lib().ref_step(int(self.kind == KIND_F16), _ptr(self.f), _ptr(self.flags),
                                   _ptr(self.solidMask), _ptr(self.lidMask), p, _ptr(force),
                                   _ptr(eps))
            else:
                if self.outflowMode not in ("dormant", "pressure"):
                    raise ValueError("outflowMode must be 'dormant' or 'pressure'")
                if self.collision not in ("reference", "kbc"):
                    raise ValueError("collision must be 'reference' or 'kbc'")
                kind = self.step_kind | (ORC_PRESSURE_OUTFLOW if self.outflowMode == "pressure"
                                         else 0) | (ORC_KBC if self.collision == "kbc" else 0)
                rc = lib().orc_step(kind, _ptr(self.f), _ptr(self.flags),
                                    _ptr(self.solidMask), _ptr(self.lidMask), p,
                                    _ptr(self.forceBuf), _ptr(eps), _ptr(self.forceField),
                                    self.threads)
                if rc != 0:
                    raise RuntimeError("orc_step rejected kind %d" % self.step_kind)
            self.stepsDone += 1

    # -- probes ---------------------------------------------------------------
    def probeMoments(self):
        if self.stepsDone % 2 != 0:
            raise RuntimeError("moments probe requires even step count")
        p = self.params(self.stepsDone)
        if self.kind == KIND_F64:
            out = np.zeros((self.N, 4), np.float64)
        else:
            out = np.zeros((self.N, 4), np.float32)
        if self.backend == "ref":
            ref_lib().ref_moments(int(self.kind == KIND_F16), _ptr(self.f), _ptr(self.flags), p,
                                  _ptr(out))
        else:
            lib().orc_moments(self.kind, _ptr(self.f), _ptr(self.flags), p,
                              _ptr(self.forceField), _ptr(out))
        return out

    def probeForce(self, xRange, yRange):
        """Two steps with the odd-pass momentum exchange; box sum in double (Sim.swift:359-372)."""
        if self.stepsDone % 2 != 0:
            raise RuntimeError("force probe requires even step count")
        if self.forceBuf is None:
            raise RuntimeError("force probe requires wantsForces")
        self.forceBuf[:] = 0
        self._force_steps = {self.stepsDone + 1}
        self.run(2)
        self._force_steps = set()
        fb = self.forceBuf.reshape(self.nz, self.ny, self.nx, 4)
        tot = np.zeros(3)
        for z in range(self.nz):
            for y in range(yRange[0], yRange[1] + 1):
                for x in range(xRange[0], xRange[1] + 1):
                    tot += fb[z, y, x, :3].astype(np.float64)
        return tot

    def kineticEnergySum(self):
        """sum over cells of |u|^2, |u|^2 formed in the storage arithmetic, summed in double."""
        m = self.probeMoments()
        if self.kind == KIND_F64:
            return float(np.sum(m[:, 0] * m[:, 0] + m[:, 1] * m[:, 1] + m[:, 2] * m[:, 2]))
        u2 = (m[:, 0] * m[:, 0] + m[:, 1] * m[:, 1]) + m[:, 2] * m[:, 2]
        return float(np.sum(u2.astype(np.float64)))

    def observables(self):
        """(sum |u|^2, sum 2 nu S:S) over fluid cells of the current state, in
        the arithmetic of the oracle's kind, summed in double (the library's
        kineticEnergySum / dissipationSum restated). Even step counts only."""
        if self.stepsDone % 2 != 0:
            raise RuntimeError("observables require an even step count")
        out = np.zeros(2)
        lib().orc_observables(self.kind, _ptr(self.f), _ptr(self.flags),
                              self.params(self.stepsDone), _ptr(self.forceField), self.omega,
                              int(self.threads), _ptr(out))
        return float(out[0]), float(out[1])

    def adjointForce(self, steps, box, direction=(1.0, 0.0, 0.0), grads=True,
                     trajectory="fp64", f0=None, threads=None, checkpoint=0):
        """FP64 adjoint of J = mean over the odd steps of direction . F_box.

        Runs the window [stepsDone, stepsDone + steps) from the current state
        (or from `f0`, 19 x N) without advancing it. `trajectory` is the forward
        the adjoint linearises about: "fp64" (the FP64 oracle), or "fp32" /
        "fp16" (FP32 arithmetic over FP32 / FP16 storage: the library's own
        forward, value for value, with the local Jacobians taken in FP64 at the
        stored states). `checkpoint`: states are recomputed from a checkpoint
        every that many steps (0 keeps all). Returns (J, dJ/deps, dJ/dF) with
        dJ/dF of shape (3, N); the gradients are None when grads=False."""
        traj = {"fp32": 0, "fp16": 1, "fp64": 2}[trajectory]
        src = self.f if f0 is None else f0
        f0 = np.ascontiguousarray(src, dtype=np.float64).reshape(19, self.N)
        if trajectory == "fp16" and not np.array_equal(f0.astype(np.float16).astype(np.float64), f0):
            raise ValueError("an FP16-storage trajectory starts from FP16 values")
        if trajectory == "fp32" and not np.array_equal(f0.astype(np.float32).astype(np.float64), f0):
            raise ValueError("an FP32-storage trajectory starts from FP32 values")
        if self.outflowMode != "dormant" or self.collision != "reference":
            raise ValueError("the oracle adjoint covers the dormant outflow wall and the "
                             "reference collision only")
        if threads is None:
            threads = os.cpu_count() or 1
        P = b"".join(self.params(self.stepsDone + t) for t in range(int(steps)))
        box = (ctypes.c_int * 4)(int(box[0][0]), int(box[0][1]), int(box[1][0]), int(box[1][1]))
        d3 = (ctypes.c_double * 3)(*[float(v) for v in direction])
        J = ctypes.c_double()
        ge = np.zeros(self.N) if grads else None
        gf = np.zeros((3, self.N)) if grads else None
        rc = lib().orc_adjoint_force_ex(traj, _ptr(f0), _ptr(self.flags), _ptr(self.solidMask),
                                        _ptr(self.lidMask), P, int(steps), _ptr(self.eps),
                                        _ptr(self.forceField), box, d3, int(threads),
                                        int(checkpoint), ctypes.byref(J), _ptr(ge), _ptr(gf))
        if rc != 0:
            raise RuntimeError("orc_adjoint_force_ex failed")
        return J.value, ge, gf

    def adjointDissipation(self, steps, every, grads=True, trajectory="fp64", f0=None,
                           threads=None, checkpoint=0):
        """FP64 adjoint of J = mean over m = 1 .. steps // every of the
        dissipation sum (2 nu S:S over fluid cells, as observables()) of the
        state after m * every steps of the window; `every` even and the window
        starting at an even step count. Arguments and returns as adjointForce."""
        traj = {"fp32": 0, "fp16": 1, "fp64": 2}[trajectory]
        if self.stepsDone % 2 != 0 or every % 2 != 0 or steps < every:
            raise ValueError("dissipation samples need even step counts and steps >= every")
        src = self.f if f0 is None else f0
        f0 = np.ascontiguousarray(src, dtype=np.float64).reshape(19, self.N)
        if self.outflowMode != "dormant" or self.collision != "reference":
            raise ValueError("the oracle adjoint covers the dormant outflow wall and the "
                             "reference collision only")
        if threads is None:
            threads = os.cpu_count() or 1
        P = b"".join(self.params(self.stepsDone + t) for t in range(int(steps)))
        J = ctypes.c_double()
        ge = np.zeros(self.N) if grads else None
        gf = np.zeros((3, self.N)) if grads else None
        rc = lib().orc_adjoint_dissipation_ex(traj, _ptr(f0), _ptr(self.flags),
                                              _ptr(self.solidMask), _ptr(self.lidMask), P,
                                              int(steps), int(every), float(self.omega),
                                              _ptr(self.eps), _ptr(self.forceField),
                                              int(threads), int(checkpoint), ctypes.byref(J),
                                              _ptr(ge), _ptr(gf))
        if rc != 0:
            raise RuntimeError("orc_adjoint_dissipation_ex failed")
        return J.value, ge, gf

    def massSum(self):
        return float(lib().orc_mass(self.kind, _ptr(self.f), self.f.size))

    @property
    def stateDigest(self):
        return hashlib.sha256(self.f.tobytes()).hexdigest()


def mesh_solid_fractions(tris, nx, ny, nz, scale, offset):
    """Restatement of meshSolidFractions (StlVoxels.swift:52-117); tris is a
    (count, 3, 3) array of mesh-space vertices."""
    t = np.ascontiguousarray(tris, dtype=np.float32).reshape(-1, 9)
    off = np.ascontiguousarray(offset, dtype=np.float32).reshape(3)
    out = np.zeros(int(nx) * int(ny) * int(nz), np.float32)
    lib().orc_mesh_solid_fractions(_ptr(t) if t.size else None, t.shape[0], nx, ny, nz,
                                   float(np.float32(scale)), _ptr(off), _ptr(out))
    return out


def colorize(moments4, flags, eps, nx, ny, z_slice, uref, backend="oracle"):
    """The |u| colormap of slice z (Kernels.metal:465-500) as an (ny, nx, 4)
    float16 RGBA image, rows as the kernel writes them (y flipped). moments4:
    (N, 4) float32 momentsEven output; flags: N uint8; eps: N float32 or None.
    backend "ref" runs the reference's own kernel source."""
    m = np.ascontiguousarray(moments4, dtype=np.float32).reshape(-1, 4)
    fl = np.ascontiguousarray(flags, dtype=np.uint8).reshape(-1)
    e = None if eps is None else np.ascontiguousarray(eps, dtype=np.float32).reshape(-1)
    out = np.zeros((int(ny), int(nx), 4), np.float16)
    if backend == "ref":
        import struct as _st
        # VizParams {nx, ny, nz, zSlice, uref, useEps, pad0, pad1}, Kernels.metal:458-463
        vp = _st.pack("<4IfI2f", nx, ny, fl.size // (nx * ny), z_slice, float(uref),
                      0 if e is None else 1, 0.0, 0.0)
        ref_lib().ref_colorize(_ptr(m), _ptr(fl), _ptr(e), vp, _ptr(out))
    else:
        lib().orc_colorize(_ptr(m), _ptr(fl), _ptr(e), nx, ny, z_slice, float(uref),
                           0 if e is None else 1, _ptr(out))
    return out
