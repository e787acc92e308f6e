"""Python host API over libmafem.so, mirroring MembraneAleFem.jl's entry points.

The names, argument meanings and error behaviour follow the reference:

=======================================  ==========================================
reference (Julia)                        here
=======================================  ==========================================
``Params(...)`` (Params.jl:36-55)        :class:`Params`
``Mesh(p; args...)`` (Mesh.jl:79)        :class:`Mesh`
``prepare_input(p; args...)``            :func:`prepare_input`
``calc_r_K(mesh, xms, cps, t, Δt, p)``   :meth:`Solver.calc_r_K`
``-K \\ r``                               :meth:`Solver.solve`
``update_xms!(...)`` (predictor)         :meth:`Solver.predict`
``time_step!(mesh, xms, cps, t, Δt, p)`` :meth:`Solver.time_step` (raises
                                         ``AssertionError`` like the reference's
                                         @assert when Newton does not converge)
``run_analysis!`` / ``solve``            :meth:`Solver.run_analysis`, :func:`solve`
=======================================  ==========================================

Every array uses the reference's layout: ``xms`` is numnp x 3 and ``cps`` numnp
x ndf (Fortran order, float64), integer maps are 1-based.  All compute runs in
CUDA kernels on the GPU; there is no CPU fallback -- without the library or a
GPU every call that computes raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmafem.so")

# enums (src/input/Enums.jl, src/input/Dof.jl) -- same numeric values
F_CAVI, F_COUE, F_POIS, F_PULL, F_BEND = 1, 2, 3, 4, 5
STATIC, EUL, LAG, ALEV, ALEVB = 1, 2, 3, 4, 5
BOTTOM, RIGHT, TOP, LEFT = 1, 2, 3, 4
SHEAR, STRETCH, MOMENT = 1, 2, 3
PLAIN_FP64, FP32_REFINE = 0, 1
LU_AUTO, LU_PANELS, LU_FULL = 0, 1, 2  # mafem_set_lu_path

OK = 0
NEWTON_NOT_CONVERGED, ZERO_PIVOT, NAN_DETECTED, REFINE_STALLED = 1, 2, 3, 4
ERR_ARG, ERR_CUDA, ERR_OOM, ERR_UNSUPPORTED, ERR_ADMISSION = -1, -2, -3, -4, -5


class MafemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class NewtonNotConverged(AssertionError):
    """The reference's ``@assert εs[end] < p.εnr`` (FiniteElement.jl:61)."""


class _CParams(C.Structure):
    _fields_ = [("motion", C.c_int32), ("scenario", C.c_int32), ("num1el", C.c_int32),
                ("num2el", C.c_int32), ("length", C.c_double), ("kb", C.c_double),
                ("kg", C.c_double), ("zeta_v", C.c_double), ("pn", C.c_double),
                ("poly", C.c_int32), ("gp1d", C.c_int32), ("nders", C.c_int32),
                ("nen", C.c_int32), ("alpha_db", C.c_double), ("alpha_m", C.c_double),
                ("eps_k", C.c_double), ("eps_nr", C.c_double)]


class _CArgs(C.Structure):
    _fields_ = [("pull_speed", C.c_double), ("bend_tm", C.c_double), ("bend_mf", C.c_double),
                ("lambda0", C.c_double), ("pull_centre", C.c_int32), ("reserved", C.c_int32)]


_P64 = C.POINTER(C.c_int64)
_PD = C.POINTER(C.c_double)


class MeshDesc(C.Structure):
    """mafem_mesh_desc (include/mafem.h)."""
    _fields_ = [("num1el", C.c_int64), ("num2el", C.c_int64), ("numel", C.c_int64),
                ("num1np", C.c_int64), ("num2np", C.c_int64), ("numnp", C.c_int64),
                ("ndf", C.c_int64), ("nmdf", C.c_int64), ("dofs", C.c_int64 * 8),
                ("IX", _P64), ("ID", _P64), ("n_uel", C.c_int64), ("uel_ids", _P64),
                ("ufns", _PD), ("bdry_n_uel", C.c_int64 * 4), ("bdry_uel_ids", _P64 * 4),
                ("bdry_ufns", _PD * 4), ("n_neu", C.c_int64), ("neu_bdry", _P64),
                ("neu_type", _P64), ("neu_val", _PD), ("n_dir", C.c_int64),
                ("dir_unknown", _P64), ("dir_node", _P64), ("dir_val", _PD)]


class StepStats(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("refine_iters", C.c_int32),
                ("eps", C.c_double * 14), ("res_norm", C.c_double * 14),
                ("ms_assemble", C.c_double), ("ms_factor", C.c_double),
                ("ms_solve", C.c_double), ("ms_total", C.c_double)]

    def as_dict(self):
        n = self.newton_iters
        return {"newton_iters": n, "refine_iters": self.refine_iters,
                "eps": list(self.eps[:n]), "res_norm": list(self.res_norm[:n]),
                "ms_assemble": self.ms_assemble, "ms_factor": self.ms_factor,
                "ms_solve": self.ms_solve, "ms_total": self.ms_total}


class _CRequest(C.Structure):
    _fields_ = [("mesh", C.c_void_p), ("params", C.c_void_p), ("args", C.c_void_p), ("precision", C.c_int32),
                ("nsteps", C.c_int32), ("t0", C.c_double), ("dt", C.c_double), ("xms0", C.c_void_p),
                ("cps0", C.c_void_p), ("refine_tol", C.c_double), ("ramp_steps", C.c_int32),
                ("reserved", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("graph_launches", C.c_int64), ("graph_captures", C.c_int64), ("graphs_cached", C.c_int64),
                ("kernel_launches", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [("steps_done", C.c_int64), ("rounds", C.c_int64), ("p50_step_ms", C.c_double),
                ("p99_step_ms", C.c_double), ("max_step_ms", C.c_double), ("bytes_in_use", C.c_int64),
                ("budget_bytes", C.c_int64), ("active", C.c_int32), ("pending", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class KernelTimes(C.Structure):
    _fields_ = [("ms_assemble", C.c_double), ("ms_panel", C.c_double), ("ms_apply", C.c_double),
                ("n_panel", C.c_int64), ("n_apply", C.c_int64), ("n", C.c_int64), ("kl", C.c_int64),
                ("ku", C.c_int64), ("nb", C.c_int64), ("ndfp", C.c_int64),
                ("flop_panel", C.c_double), ("flop_apply", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """Load libmafem.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run membranealefem.jl_gb300/build.py "
                              "(the CUDA library is required; there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.mafem_last_error.restype = C.c_char_p
        L.mafem_last_error.argtypes = [vp]
        L.mafem_mesh_build.argtypes = [C.POINTER(_CParams), C.POINTER(_CArgs), C.POINTER(vp)]
        L.mafem_mesh_view.argtypes = [vp, C.POINTER(MeshDesc)]
        L.mafem_mesh_free.argtypes = [vp]
        L.mafem_mesh_free.restype = None
        L.mafem_prepare_input.argtypes = [vp, C.POINTER(_CParams), _PD, _PD]
        L.mafem_mesh_half_bandwidth.argtypes = [C.POINTER(MeshDesc)]
        L.mafem_mesh_half_bandwidth.restype = C.c_int64
        L.mafem_create.argtypes = [C.POINTER(MeshDesc), C.POINTER(_CParams), C.POINTER(_CArgs),
                                   C.c_int32, C.POINTER(vp)]
        L.mafem_destroy.argtypes = [vp]
        L.mafem_device_bytes.argtypes = [vp]
        L.mafem_device_bytes.restype = C.c_int64
        L.mafem_footprint_bytes.argtypes = [C.POINTER(MeshDesc), C.c_int32]
        L.mafem_footprint_bytes.restype = C.c_int64
        L.mafem_upload_state.argtypes = [vp, _PD, _PD]
        L.mafem_download_state.argtypes = [vp, _PD, _PD]
        L.mafem_calc_r_K.argtypes = [vp, C.c_double, C.c_double, _PD, _PD, C.c_int64]
        L.mafem_solve.argtypes = [vp, _PD, _PD]
        L.mafem_predict.argtypes = [vp, C.c_double]
        L.mafem_time_step.argtypes = [vp, C.c_double, C.c_double, C.POINTER(StepStats)]
        L.mafem_time_step_host.argtypes = [vp, _PD, _PD, C.c_double, C.c_double,
                                           C.POINTER(StepStats)]
        L.mafem_run.argtypes = [vp, _PD, C.c_int32, C.c_double, C.POINTER(StepStats)]
        L.mafem_launch_count.argtypes = [vp]
        L.mafem_launch_count.restype = C.c_int64
        L.mafem_set_lu_path.argtypes = [vp, C.c_int32]
        L.mafem_set_patch_ctas.argtypes = [vp, C.c_int32]
        L.mafem_autotune_patch.argtypes = [vp]
        L.mafem_set_refinement.argtypes = [vp, C.c_int32, C.c_double]
        L.mafem_set_wait_test.argtypes = [vp, C.c_int32, C.c_int32]
        L.mafem_set_dirichlet_scale.argtypes = [vp, C.c_double]
        L.mafem_solve_band.argtypes = [vp, _PD, C.c_int64, _PD, _PD]
        L.mafem_fallback_count.argtypes = [vp]
        L.mafem_fallback_count.restype = C.c_int64
        L.mafem_trace_patch_solve.argtypes = [vp, C.c_double, C.c_double, C.POINTER(C.c_int64), C.c_int64]
        L.mafem_pull_force.argtypes = [vp, _PD]
        L.mafem_pull_position.argtypes = [vp, _PD]
        L.mafem_format_double.argtypes = [C.c_double, C.c_char_p, C.c_int32]
        L.mafem_writedlm.argtypes = [C.c_char_p, _PD, C.c_int64, C.c_int64]
        L.mafem_readdlm.argtypes = [C.c_char_p, _PD, C.c_int64, C.c_int64]
        L.mafem_write_state.argtypes = [vp, C.c_char_p, C.c_int64]
        L.mafem_write_state_async.argtypes = [vp, C.c_int32, C.c_char_p, C.c_int64]
        L.mafem_flush_state_writes.argtypes = [vp]
        L.mafem_read_state.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.mafem_snapshot_reserve.argtypes = [vp, C.c_int32]
        L.mafem_snapshot.argtypes = [vp, C.c_int32]
        L.mafem_restore.argtypes = [vp, C.c_int32]
        L.mafem_set_launch_ctas.argtypes = [vp, C.c_int32]
        L.mafem_batch_create.argtypes = [C.POINTER(vp), C.c_int32, C.c_int32, C.POINTER(vp)]
        L.mafem_batch_step.argtypes = [vp, _PD, _PD, C.POINTER(C.c_int32), C.POINTER(StepStats)]
        L.mafem_batch_destroy.argtypes = [vp]
        L.mafem_batch_set_patch_solve.argtypes = [vp, C.c_int32]
        L.mafem_batch_set_rounds.argtypes = [vp, C.c_int32, C.c_int32]
        L.mafem_tangent_tile.argtypes = [vp, C.POINTER(C.c_int32), _PD, _PD]
        L.mafem_batch_get_stats.argtypes = [vp, C.POINTER(BatchStats)]
        L.mafem_server_create.argtypes = [C.c_int64, C.c_int32, C.POINTER(vp)]
        L.mafem_server_destroy.argtypes = [vp]
        L.mafem_server_submit.argtypes = [vp, C.POINTER(_CRequest), C.POINTER(C.c_int64)]
        L.mafem_server_round.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.mafem_server_result.argtypes = [vp, C.c_int64, _PD, _PD, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.mafem_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
        L.mafem_profile_factor.argtypes = [vp, C.c_double, C.c_double, C.POINTER(KernelTimes)]
        L.mafem_probe_fp64_tflops.argtypes = [C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_PD)


def _raise(rc: int, h=None):
    if rc == OK:
        return
    msg = lib().mafem_last_error(h).decode()
    if rc == NEWTON_NOT_CONVERGED:
        raise NewtonNotConverged(msg)
    raise MafemError(rc, msg)


# ---- state files (src/Analysis.jl:75-78, src/Input.jl:35-37) -------------------------

F_PULL_HEADER = "time\txp\typ\tzp\tfx\tfy\tfz"  # first line of f-pull.txt (Analysis.jl:52-54)


def format_double(x: float) -> str:
    """Julia's print(::Float64): shortest round-trip digits, "1.0", "1.0e-5", "1.0e6"."""
    buf = C.create_string_buffer(32)
    n = lib().mafem_format_double(float(x), buf, 32)
    if n < 0:
        raise MafemError(n, "format_double")
    return buf.value.decode()


def writedlm(path: str, a) -> None:
    """DelimitedFiles.writedlm of a Float64 matrix (tab-separated rows)."""
    a = np.asfortranarray(np.atleast_2d(np.asarray(a, dtype=np.float64)))
    _raise(lib().mafem_writedlm(os.fsencode(path), _dp(a), a.shape[0], a.shape[1]))


def readdlm(path: str, rows: int, cols: int) -> np.ndarray:
    """DelimitedFiles.readdlm of a rows x cols Float64 matrix (the shape is checked)."""
    a = np.zeros((rows, cols), order="F")
    _raise(lib().mafem_readdlm(os.fsencode(path), _dp(a), rows, cols))
    return a


def state_files(dir_: str, t_id: int) -> tuple[str, str]:
    """The names run_analysis! writes: <dir>/t<t_id>-xms.txt, <dir>/t<t_id>-cps.txt."""
    return (os.path.join(dir_, f"t{t_id}-xms.txt"), os.path.join(dir_, f"t{t_id}-cps.txt"))


def f_pull_line(rec) -> str:
    """One line of f-pull.txt (Analysis.jl:86-90): time, x_pull[3], f_pull[3]."""
    return "\t".join(format_double(v) for v in rec)


@dataclass
class Params:
    """``Params`` (src/input/Params.jl:36-55) plus the keyword arguments the hot
    path reads (``pull_speed``, ``bend_tm``, ``bend_mf``) and two F_PULL
    extensions with no reference keyword: ``lambda0`` (edge tension and initial
    λ; 0 = the reference's kb / 4) and ``pull_centre`` (1 = pull the centre
    element (floor(n1/2) + 1, floor(n2/2) + 1) instead of ceil(numel / 2))."""

    motion: int = ALEVB
    scenario: int = F_PULL
    num1el: int = 17
    num2el: int = 17
    output: bool = False
    length: float = 64.0
    kb: float = 1.0
    kg: float = -0.5
    zeta_v: float = 1.0
    pn: float = 0.0
    poly: int = 2
    gp1d: int = 3
    nders: int = 2
    nen: int = 9
    alpha_db: float | None = None  # default length^2 (Params.jl:51)
    alpha_m: float = 1.0
    eps_k: float = 1e-15
    eps_nr: float = 1e-12
    pull_speed: float = 0.0
    bend_tm: float = 1.0
    bend_mf: float = 0.0
    lambda0: float = 0.0
    pull_centre: int = 0

    def c_params(self) -> _CParams:
        adb = self.length ** 2 if self.alpha_db is None else self.alpha_db
        return _CParams(self.motion, self.scenario, self.num1el, self.num2el, self.length,
                        self.kb, self.kg, self.zeta_v, self.pn, self.poly, self.gp1d, self.nders,
                        self.nen, adb, self.alpha_m, self.eps_k, self.eps_nr)

    def c_args(self) -> _CArgs:
        return _CArgs(self.pull_speed, self.bend_tm, self.bend_mf, self.lambda0, self.pull_centre, 0)


class Mesh:
    """``Mesh(p; args...)`` built by the library (src/input/Mesh.jl:94-302)."""

    def __init__(self, p: Params):
        self.p = p
        self._cp, self._ca = p.c_params(), p.c_args()
        h = C.c_void_p()
        _raise(lib().mafem_mesh_build(C.byref(self._cp), C.byref(self._ca), C.byref(h)))
        self.h = h
        self.desc = MeshDesc()
        _raise(lib().mafem_mesh_view(self.h, C.byref(self.desc)))
        d = self.desc
        (self.num1el, self.num2el, self.numel, self.num1np, self.num2np, self.numnp, self.ndf,
         self.nmdf) = (d.num1el, d.num2el, d.numel, d.num1np, d.num2np, d.numnp, d.ndf, d.nmdf)
        self.dofs = [int(v) for v in d.dofs]
        self.half_bw = int(lib().mafem_mesh_half_bandwidth(C.byref(d)))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().mafem_mesh_free(self.h)
        except Exception:
            pass

    def _arr(self, ptr, n, dtype):
        return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)

    @property
    def IX(self):
        return self._arr(self.desc.IX, 9 * self.numel, np.int64).reshape(self.numel, 9).T

    @property
    def ID(self):
        return self._arr(self.desc.ID, self.ndf * self.numnp, np.int64).reshape(self.numnp, self.ndf).T

    @property
    def LM(self):
        """``reshape(ID[:, IX], ndf*NEN, numel)`` (Mesh.jl:299)."""
        ID, IX = self.ID, self.IX
        return ID[:, IX.T.reshape(-1) - 1].T.reshape(self.numel, 9 * self.ndf).T

    @property
    def ID_inv(self):
        """(node, dof) of each unknown, 1-based (Mesh.jl:291-296)."""
        ID = self.ID
        nodes, dofs = np.nonzero(ID.T)
        order = np.argsort(ID.T[nodes, dofs])
        return np.stack([nodes[order] + 1, dofs[order] + 1], axis=1)

    def area_tables(self):
        uel = self._arr(self.desc.uel_ids, self.numel, np.int64)
        uf = self._arr(self.desc.ufns, self.desc.n_uel * 9 * 55, np.float64)
        return uel, uf.reshape(self.desc.n_uel, 9, 55)

    def bdry_tables(self, b: int):
        k = b - 1
        nel = self.num1el if b in (BOTTOM, TOP) else self.num2el
        uel = self._arr(self.desc.bdry_uel_ids[k], nel, np.int64)
        nu = self.desc.bdry_n_uel[k]
        uf = self._arr(self.desc.bdry_ufns[k], nu * 3 * 55, np.float64)
        return uel, uf.reshape(nu, 3, 55)

    def neumann(self):
        d = self.desc
        return [(int(d.neu_bdry[k]), int(d.neu_type[k]), float(d.neu_val[k])) for k in range(d.n_neu)]

    def dirichlet(self):
        d = self.desc
        return [(int(d.dir_unknown[k]), int(d.dir_node[k]), float(d.dir_val[k])) for k in range(d.n_dir)]


def prepare_input(p: Params, mesh: Mesh | None = None):
    """``prepare_input(p; args...)`` (src/Input.jl:22-121): mesh, xms, cps."""
    mesh = mesh or Mesh(p)
    xms = np.zeros((mesh.numnp, 3), order="F")
    cps = np.zeros((mesh.numnp, mesh.ndf), order="F")
    _raise(lib().mafem_prepare_input(mesh.h, C.byref(mesh._cp), _dp(xms), _dp(cps)))
    return mesh, xms, cps


def footprint_bytes(mesh: Mesh, precision: int = PLAIN_FP64) -> int:
    return int(lib().mafem_footprint_bytes(C.byref(mesh.desc), precision))


class Solver:
    """Device-resident state of one patch: the replacement of ``calc_r_K`` + ``\\``
    and of ``time_step!`` (src/analysis/FiniteElement.jl:11-200)."""

    def __init__(self, mesh: Mesh, p: Params | None = None, precision: int = PLAIN_FP64,
                 desc: MeshDesc | None = None):
        self.mesh = mesh
        self.p = p or mesh.p
        self.precision = precision
        self._cp, self._ca = self.p.c_params(), self.p.c_args()
        self.desc = desc or mesh.desc
        h = C.c_void_p()
        _raise(lib().mafem_create(C.byref(self.desc), C.byref(self._cp), C.byref(self._ca),
                                  precision, C.byref(h)))
        self.h = h
        self.nmdf = self.desc.nmdf
        self.kl = mesh.half_bw if mesh is not None else int(
            lib().mafem_mesh_half_bandwidth(C.byref(self.desc)))

    def close(self):
        if getattr(self, "h", None):
            lib().mafem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def device_bytes(self) -> int:
        return int(lib().mafem_device_bytes(self.h))

    def launch_count(self) -> int:
        """Kernels this handle has enqueued so far."""
        return int(lib().mafem_launch_count(self.h))

    def pull_force(self) -> np.ndarray:
        """calc_pull_force (PullForce.jl:61-80) on the resident state: 3-vector."""
        f = np.zeros(3)
        _raise(lib().mafem_pull_force(self.h, _dp(f)), self.h)
        return f

    def pull_position(self) -> np.ndarray:
        """x_pull (Analysis.jl:83-84): mean position of the pull element's nine nodes."""
        x = np.zeros(3)
        _raise(lib().mafem_pull_position(self.h, _dp(x)), self.h)
        return x

    def pull_record(self, time: float) -> list:
        """The f-pull.txt record of run_analysis! (Analysis.jl:81-91) at `time`."""
        return [float(time), *self.pull_position(), *self.pull_force()]

    def write_state(self, dir_: str, t_id: int) -> None:
        """writedlm of xms / cps to <dir>/t<t_id>-{xms,cps}.txt; waits for the files."""
        _raise(lib().mafem_write_state(self.h, os.fsencode(dir_), t_id), self.h)

    def write_state_async(self, dir_: str, t_id: int, slot: int = -1) -> None:
        """Queue the same files (of the state, or of snapshot `slot`) for the library's
        writer thread; the copy is ordered after the steps already enqueued."""
        _raise(lib().mafem_write_state_async(self.h, slot, os.fsencode(dir_), t_id), self.h)

    def flush_state_writes(self) -> None:
        _raise(lib().mafem_flush_state_writes(self.h), self.h)

    def read_state(self, xms_file: str, cps_file: str) -> None:
        """readdlm both files into the resident state (restart, MembraneAleFem.jl:75-107)."""
        _raise(lib().mafem_read_state(self.h, os.fsencode(xms_file), os.fsencode(cps_file)), self.h)

    def snapshot_reserve(self, nslots: int) -> None:
        _raise(lib().mafem_snapshot_reserve(self.h, nslots), self.h)

    def snapshot(self, slot: int) -> None:
        """Copy the state into device snapshot `slot` (stream-ordered, does not wait)."""
        _raise(lib().mafem_snapshot(self.h, slot), self.h)

    def restore(self, slot: int) -> None:
        """Copy device snapshot `slot` back into the state (stream-ordered)."""
        _raise(lib().mafem_restore(self.h, slot), self.h)

    def set_launch_ctas(self, ctas: int) -> int:
        """CTAs of the persistent factorisation (0: all SMs); returns the value in use."""
        return int(lib().mafem_set_launch_ctas(self.h, ctas))

    def set_refinement(self, max_sweeps: int = 30, tol: float = 1e-10) -> None:
        """FP32 form: refinement tolerance (|r - A x| <= tol |r| alone; last correction
        <= tol |x| in the batched solve) and sweep cap."""
        _raise(lib().mafem_set_refinement(self.h, max_sweeps, tol), self.h)

    def trace_patch_solve(self, time: float, dt: float):
        """FP32 form: per-panel phase stamps (ns) of the batched one-CTA factorisation
        of the resident state, as an (npan, 6) array, and the factor / refine kernel
        times in ms."""
        cap = 6 * 4096 + 182
        buf = (C.c_int64 * cap)()
        npan = lib().mafem_trace_patch_solve(self.h, time, dt, buf, cap)
        _raise(0 if npan >= 0 else npan, self.h)
        a = np.ctypeslib.as_array(buf)[: 6 * npan + 182].copy()
        self.last_refine_trace = a[6 * npan + 2: 6 * npan + 130].reshape(32, 4)
        self.last_solve_phases = a[6 * npan + 130: 6 * npan + 146]
        self.last_refine_residuals = a[6 * npan + 146: 6 * npan + 178].view(np.float64)
        self.last_refine_status = (int(a[6 * npan + 180]), int(a[6 * npan + 181]))
        return a[: 6 * npan].reshape(npan, 6), a[6 * npan] / 1e6, a[6 * npan + 1] / 1e6

    def solve_band(self, band, rhs):
        """x with K x = rhs for a caller's band K (LAPACK layout of calc_r_K's band,
        ldab >= 3 kl + 1) through this handle's factorisation and solves."""
        band = np.ascontiguousarray(band, dtype=np.float64)  # row j = band column j
        rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        x = np.zeros(self.nmdf)
        _raise(lib().mafem_solve_band(self.h, _dp(band), band.shape[1], _dp(rhs), _dp(x)), self.h)
        return x

    def set_dirichlet_scale(self, scale: float) -> None:
        """Inhomogeneous Dirichlet entries of the resident state = scale x their
        values (stream-ordered before the next step): a ramped pull."""
        _raise(lib().mafem_set_dirichlet_scale(self.h, float(scale)), self.h)

    def fallback_count(self) -> int:
        """Factorisations redone with full partial pivoting so far."""
        return int(lib().mafem_fallback_count(self.h))

    def set_wait_test(self, limit_polls: int = 0, withhold_panel: int = -1) -> None:
        """Failure-detection test hook (mafem_set_wait_test): bounded inter-CTA waits
        give up after limit_polls polls; the back substitution withholds the flag of
        the panel withhold_panel places before the last.  (0, -1) restores the default."""
        _raise(lib().mafem_set_wait_test(self.h, limit_polls, withhold_panel), self.h)

    def set_lu_path(self, path: int) -> None:
        """Select the banded LU: LU_AUTO (default), LU_PANELS or LU_FULL."""
        _raise(lib().mafem_set_lu_path(self.h, path), self.h)

    def set_patch_ctas(self, ctas: int) -> None:
        """Batched FP32 form: CTAs (1, 2 or 4) of the cluster that factors this
        patch; 0 chooses by band width."""
        _raise(lib().mafem_set_patch_ctas(self.h, ctas), self.h)

    def autotune_patch(self) -> None:
        """Measure (once per device and patch shape) the batched FP32 factorisation
        of this patch on 1, 2 and 4 CTAs for the round-by-round autotuner; call
        between steps with the GPU otherwise idle."""
        _raise(lib().mafem_autotune_patch(self.h), self.h)

    def tangent_tile(self):
        """The batched rounds' FP32 tangent kernel for this kind of patch:
        (elements per CTA chosen, ms with 2, ms with 4), or None before a batch
        or server has measured it."""
        e = C.c_int32()
        m2, m4 = C.c_double(), C.c_double()
        rc = lib().mafem_tangent_tile(self.h, C.byref(e), C.byref(m2), C.byref(m4))
        if rc == ERR_UNSUPPORTED:
            return None
        _raise(rc, self.h)
        return int(e.value), float(m2.value), float(m4.value)

    def profile_factor(self, time: float, dt: float) -> dict:
        """Per-kernel device time of one assembly + factorisation of the resident state."""
        kt = KernelTimes()
        _raise(lib().mafem_profile_factor(self.h, time, dt, C.byref(kt)), self.h)
        return kt.as_dict()

    def upload(self, xms, cps):
        xms = np.asfortranarray(xms, dtype=np.float64)
        cps = np.asfortranarray(cps, dtype=np.float64)
        _raise(lib().mafem_upload_state(self.h, _dp(xms), _dp(cps)), self.h)

    def download(self):
        xms = np.zeros((self.desc.numnp, 3), order="F")
        cps = np.zeros((self.desc.numnp, self.desc.ndf), order="F")
        _raise(lib().mafem_download_state(self.h, _dp(xms), _dp(cps)), self.h)
        return xms, cps

    def calc_r_K(self, xms, cps, time: float, dt: float, tangent: bool = True):
        """r (nmdf) and K in LAPACK band layout ((nmdf, 3kl+1): row j holds column j,
        A(i, j) at [j, 2kl + i - j]); state is uploaded first."""
        self.upload(xms, cps)
        r = np.zeros(self.nmdf)
        kl = self.kl
        ldab = 3 * kl + 1
        ab = np.zeros((self.nmdf, ldab)) if tangent else None
        _raise(lib().mafem_calc_r_K(self.h, time, dt, _dp(r), _dp(ab) if tangent else None, ldab),
               self.h)
        return r, ab

    def solve(self, r):
        """Δu = -K \\ r for the K of the last calc_r_K (FiniteElement.jl:38)."""
        r = np.ascontiguousarray(r, dtype=np.float64)
        du = np.zeros(self.nmdf)
        _raise(lib().mafem_solve(self.h, _dp(r), _dp(du)), self.h)
        return du

    def predict(self, dt: float):
        _raise(lib().mafem_predict(self.h, dt), self.h)

    def time_step(self, xms, cps, time: float, dt: float):
        """``time_step!`` with host arrays, updated in place (Fortran-ordered)."""
        assert xms.flags.f_contiguous and cps.flags.f_contiguous
        assert xms.dtype == np.float64 and cps.dtype == np.float64
        st = StepStats()
        rc = lib().mafem_time_step_host(self.h, _dp(xms), _dp(cps), time, dt, C.byref(st))
        self.last_stats = st.as_dict()
        _raise(rc, self.h)
        return self.last_stats

    def time_step_resident(self, time: float, dt: float):
        st = StepStats()
        rc = lib().mafem_time_step(self.h, time, dt, C.byref(st))
        self.last_stats = st.as_dict()
        _raise(rc, self.h)
        return self.last_stats

    def run_analysis(self, dts, t0: float = 0.0):
        """``run_analysis!``'s time loop on the resident state (Analysis.jl:60-93)."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        st = StepStats()
        rc = lib().mafem_run(self.h, _dp(dts), len(dts), t0, C.byref(st))
        self.last_stats = st.as_dict()
        _raise(rc, self.h)
        return self.last_stats


class Batch:
    """Many patches (Solver objects, any sizes, motions and precisions) stepped
    together: each step is predictor + time_step! for every patch, their Newton
    iterations interleaved on the GPU (mafem_batch_*).  Results equal each
    Solver stepped alone.  The Solvers stay owned by the caller."""

    def __init__(self, solvers, ctas: int = 0):
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(self.solvers))(*[s.h for s in self.solvers])
        self.b = C.c_void_p()
        _raise(lib().mafem_batch_create(arr, len(self.solvers), ctas, C.byref(self.b)))

    def set_patch_solve(self, on: bool) -> bool:
        """Batched one-CTA-per-patch FP32 solve for the FP32 patches (default on);
        returns whether it is in use."""
        rc = lib().mafem_batch_set_patch_solve(self.b, int(on))
        if rc < 0:
            _raise(rc)
        return rc == 1

    def set_rounds(self, batched_assembly: bool = True, graphs: bool = True):
        """Newton rounds of the batched-solve patches: one launch per kernel for
        all of them (default on), replayed from CUDA graphs (default on)."""
        _raise(lib().mafem_batch_set_rounds(self.b, int(batched_assembly), int(graphs)))

    def stats(self) -> dict:
        """Graph replays and captures, graphs held, kernels enqueued."""
        st = BatchStats()
        _raise(lib().mafem_batch_get_stats(self.b, C.byref(st)))
        return st.as_dict()

    def step(self, times, dts):
        """One time step of every patch; returns (statuses, list of step-stat dicts).
        Each patch's outcome, failures included, is its status; an error of the
        call itself (a code no patch reports) raises."""
        n = len(self.solvers)
        times = np.ascontiguousarray(np.broadcast_to(times, (n,)), dtype=np.float64)
        dts = np.ascontiguousarray(np.broadcast_to(dts, (n,)), dtype=np.float64)
        status = (C.c_int32 * n)()
        stats = (StepStats * n)()
        rc = lib().mafem_batch_step(self.b, _dp(times), _dp(dts), status, stats)
        statuses = [int(x) for x in status]
        if rc != OK and rc not in statuses:
            _raise(rc)
        return statuses, [st.as_dict() for st in stats]

    def close(self):
        if self.b:
            lib().mafem_batch_destroy(self.b)
            self.b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def solve(p: Params, dts, t0: float = 0.0, precision: int = PLAIN_FP64, xms=None, cps=None):
    """``solve(p; args...)`` (src/MembraneAleFem.jl:44-60) without file output:
    returns (mesh, xms, cps) after the time steps ``dts``."""
    mesh, x0, c0 = prepare_input(p)
    xms = x0 if xms is None else np.asfortranarray(xms, dtype=np.float64)
    cps = c0 if cps is None else np.asfortranarray(cps, dtype=np.float64)
    with Solver(mesh, p, precision) as s:
        s.upload(xms, cps)
        s.run_analysis(dts, t0)
        xms, cps = s.download()
    return mesh, xms, cps


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n uniform doubles in [0, 1) from SplitMix64 (portable, seedable)."""
    out = np.empty(n, dtype=np.float64)
    with np.errstate(over="ignore"):
        s = np.uint64(seed)
        for i in range(n):
            s = s + np.uint64(0x9E3779B97F4A7C15)
            z = s
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
            out[i] = float(z >> np.uint64(11)) * (1.0 / 9007199254740992.0)
    return out


def perturb_interior_z(mesh: Mesh, xms: np.ndarray, seed: int = 0, amp: float = 1e-4) -> np.ndarray:
    """Seeded out-of-plane perturbation z ~ U[-amp, amp] of the nodes not on the
    outer boundary (the synthetic initial state of the benchmark workloads)."""
    u = splitmix64(seed, mesh.numnp)
    s1 = np.arange(mesh.numnp) % mesh.num1np
    s2 = np.arange(mesh.numnp) // mesh.num1np
    interior = (s1 > 0) & (s1 < mesh.num1np - 1) & (s2 > 0) & (s2 < mesh.num2np - 1)
    xms[:, 2] += np.where(interior, amp * (2.0 * u - 1.0), 0.0)
    return xms


class Server:
    """Continuous batching of many solves (mafem_server_*): submit requests
    (patch, initial state, number of steps), call round() repeatedly; each round
    admits what fits the HBM budget and runs one Newton iteration of every
    admitted request.  result(id) returns (status, xms, cps) once a request has
    finished, None while it is queued or running."""

    def __init__(self, hbm_budget_bytes: int = 0, max_active: int = 0):
        self.s = C.c_void_p()
        _raise(lib().mafem_server_create(int(hbm_budget_bytes), int(max_active), C.byref(self.s)))
        self._keep = {}  # id -> objects the library reads until the request is admitted

    def submit(self, mesh, p, xms, cps, nsteps: int, dt: float, t0: float = 0.0,
               precision: int = FP32_REFINE, refine_tol: float = 0.0, ramp_steps: int = 0) -> int:
        xms = np.asfortranarray(xms, dtype=np.float64)
        cps = np.asfortranarray(cps, dtype=np.float64)
        cp, ca = p.c_params(), p.c_args()
        req = _CRequest(C.addressof(mesh.desc), C.addressof(cp), C.addressof(ca), precision, int(nsteps),
                        float(t0), float(dt), xms.ctypes.data, cps.ctypes.data, float(refine_tol),
                        int(ramp_steps), 0)
        rid = C.c_int64()
        _raise(lib().mafem_server_submit(self.s, C.byref(req), C.byref(rid)))
        self._keep[rid.value] = (mesh, cp, ca, (mesh.numnp, mesh.ndf))
        return rid.value

    def round(self):
        """One round; returns (active, pending)."""
        a, q = C.c_int32(), C.c_int32()
        _raise(lib().mafem_server_round(self.s, C.byref(a), C.byref(q)))
        return a.value, q.value

    def result(self, rid: int):
        mesh, _, _, (numnp, ndf) = self._keep[rid]
        xms = np.zeros((numnp, 3), order="F")
        cps = np.zeros((numnp, ndf), order="F")
        st, steps = C.c_int32(), C.c_int32()
        rc = lib().mafem_server_result(self.s, rid, _dp(xms), _dp(cps), C.byref(st), C.byref(steps))
        if rc == 1:
            return None
        _raise(rc)
        del self._keep[rid]
        return st.value, xms, cps

    def stats(self) -> dict:
        out = ServerStats()
        _raise(lib().mafem_server_get_stats(self.s, C.byref(out)))
        return out.as_dict()

    def close(self):
        if self.s:
            lib().mafem_server_destroy(self.s)
            self.s = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
