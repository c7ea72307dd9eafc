"""ctypes binding of the C ABI in ``include/sdm_capi.h``.

The shared library is the in-tree ``libsdm_gb300.so`` built by
``openmm_sdm_plugin_gb300.build``.  There is no fallback: if the library is
missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdm_gb300.so")

# status codes
SDM_OK = 0
SDM_ERR_INVALID_ARGUMENT = 1
SDM_ERR_CUDA = 2
SDM_ERR_NO_DEVICE = 3
SDM_ERR_OVERFLOW = 4
SDM_ERR_CAPACITY = 5
SDM_ERR_UNKNOWN_METHOD = 6
SDM_ERR_TIMEOUT = 7

# device status bits (sdm_check_status, results[:, R_STATUS])
DEV_FORCE_OVERFLOW, DEV_ENERGY_NONFINITE, DEV_EXCL_OVERFLOW, DEV_LIST_OVERFLOW, DEV_COORD_NONFINITE = 1, 2, 4, 8, 16

NPARAMS = 22
NRESULTS = 16
RESULT_FIELDS = ("U0", "U1", "u", "BindE", "fp", "W", "dW", "s", "E_pot", "dWdlambda",
                 "lambda1", "lambda2", "u0", "w0", "status", "nclusters")
(R_U0, R_U1, R_U, R_BINDE, R_FP, R_W, R_DW, R_S, R_EPOT, R_DWDL, R_L1, R_L2, R_U0P, R_W0P,
 R_STATUS, R_NCL) = range(16)

(OPT_GRAPH, OPT_PROFILE, OPT_SPLIT, OPT_CTAS_PER_SM, OPT_VERIFY, OPT_PAIR_RESIDENT, OPT_ZERO_COPY,
 OPT_STAGE_CHUNK, OPT_OVERLAP, OPT_LIST_GROUP) = range(10)

EXPORTED = ("sdm_create", "sdm_destroy", "sdm_last_error", "sdm_num_replicas",
            "sdm_set_displacement", "sdm_set_params", "sdm_evaluate", "sdm_evaluate_device",
            "sdm_get_state_forces", "sdm_get_state_forces_device", "sdm_check_status", "sdm_set_option", "sdm_get_option",
            "sdm_get_kernel_times", "sdm_autotune", "sdm_autotune_cached", "sdm_tune_key",
            "sdm_count_pairs", "sdm_get_grid",
            "sdm_export_lists", "sdm_evaluate_noalloc", "sdm_set_particle_params",
            "sdm_adjoint", "sdm_adjoint_device", "sdm_backward_device", "sdm_get_num_perturbed", "sdm_set_langevin", "sdm_langevin_step", "sdm_set_restraints",
            "sdm_set_restraint_control", "sdm_get_restraint_energies", "sdm_set_rigid_waters",
            "sdm_gather_positions", "sdm_scatter_forces_fixed", "sdm_evaluate_engine", "sdm_get_last_results")

NB_REACTION_FIELD, NB_PME = 0, 1
NOALLOC_MAX_PARTICLES = 8192
NOALLOC_SCRATCH_BYTES = 727296


class SdmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"sdm status {status}: {message}")
        self.status = status


class TuneResult(C.Structure):
    _fields_ = [("stage_chunk", C.c_int), ("ctas_per_sm", C.c_int), ("split", C.c_int), ("ms", C.c_float),
                ("from_cache", C.c_int), ("list_group", C.c_int), ("overlap", C.c_int)]


class SystemDesc(C.Structure):
    _fields_ = [
        ("num_particles", C.c_int),
        ("charge", C.POINTER(C.c_double)),
        ("sigma", C.POINTER(C.c_double)),
        ("epsilon", C.POINTER(C.c_double)),
        ("num_exclusions", C.c_int),
        ("exclusions", C.POINTER(C.c_int)),
        ("displacement", C.POINTER(C.c_double)),
        ("box", C.c_double * 3),
        ("cutoff", C.c_double),
        ("reaction_field_dielectric", C.c_double),
        ("num_replicas", C.c_int),
        ("num_exceptions", C.c_int),
        ("exception_pairs", C.POINTER(C.c_int)),
        ("exception_params", C.POINTER(C.c_double)),
        ("nonbonded_method", C.c_int),
        ("ewald_tolerance", C.c_double),
        ("pme_grid", C.c_int * 3),
    ]


_lock = threading.Lock()
_lib = None


def _stream(stream: int):
    """A torch ``cuda_stream`` value as the ABI's stream argument: torch's
    default stream has the handle 0, which is CUDA's legacy default stream
    (cudaStreamLegacy), not the ABI's NULL (the handle's own stream, which is
    not ordered with the caller's default-stream work)."""
    return C.c_void_p(stream if stream else 1)


def load_library(path: str = LIB_PATH):
    """Loads (once) and returns the CDLL with argument types declared."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(f"CUDA library {path} is missing: run openmm_sdm_plugin_gb300.build.build()")
        L = C.CDLL(path)
        vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
        L.sdm_create.argtypes = [C.POINTER(SystemDesc), C.c_int, C.c_int, C.POINTER(vp)]
        L.sdm_destroy.argtypes = [vp]
        L.sdm_last_error.argtypes = [vp]
        L.sdm_last_error.restype = C.c_char_p
        L.sdm_num_replicas.argtypes = [vp, ip]
        L.sdm_set_displacement.argtypes = [vp, C.c_int, vp]
        L.sdm_set_params.argtypes = [vp, C.c_int, vp]
        L.sdm_evaluate.argtypes = [vp, vp, vp, vp]
        L.sdm_evaluate_device.argtypes = [vp, vp, vp, vp, vp]
        L.sdm_get_state_forces.argtypes = [vp, vp, vp, C.c_int]
        L.sdm_get_state_forces_device.argtypes = [vp, vp, vp, vp]
        L.sdm_gather_positions.argtypes = [vp, vp, C.c_int, vp, C.c_int, vp, vp]
        L.sdm_scatter_forces_fixed.argtypes = [vp, vp, C.c_int, C.c_int, vp, vp]
        L.sdm_evaluate_engine.argtypes = [vp, vp, vp, C.c_int, vp, C.c_int, vp, vp, vp]
        L.sdm_get_last_results.argtypes = [vp, vp]
        L.sdm_check_status.argtypes = [vp, ip]
        L.sdm_set_option.argtypes = [vp, C.c_int, C.c_int]
        L.sdm_get_option.argtypes = [vp, C.c_int, ip]
        L.sdm_get_kernel_times.argtypes = [vp, C.POINTER(C.c_char_p), C.POINTER(C.c_float), ip]
        L.sdm_autotune.argtypes = [vp, vp, ip, ip]
        L.sdm_autotune_cached.argtypes = [vp, vp, C.c_char_p, C.POINTER(TuneResult)]
        L.sdm_tune_key.argtypes = [C.POINTER(SystemDesc), C.c_int, C.c_int, C.c_char_p, C.c_int]
        L.sdm_count_pairs.argtypes = [vp, vp, vp]
        L.sdm_get_grid.argtypes = [vp, C.c_int, ip]
        L.sdm_export_lists.argtypes = [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp, ip, vp, vp, vp]
        L.sdm_evaluate_noalloc.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, C.c_double,
                                           C.c_double, vp, vp, vp, vp]
        L.sdm_set_particle_params.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp]
        L.sdm_adjoint.argtypes = [vp, vp]
        L.sdm_adjoint_device.argtypes = [vp, vp, vp]
        L.sdm_get_num_perturbed.argtypes = [vp, ip]
        L.sdm_set_langevin.argtypes = [vp, C.POINTER(LangevinParams), C.c_ulonglong]
        L.sdm_langevin_step.argtypes = [vp, vp, vp, vp, vp, vp, C.c_int, vp]
        L.sdm_set_restraints.argtypes = [vp, C.c_int, C.POINTER(RestraintDesc)]
        L.sdm_set_restraint_control.argtypes = [vp, C.c_int, C.c_double]
        L.sdm_get_restraint_energies.argtypes = [vp, vp]
        L.sdm_set_rigid_waters.argtypes = [vp, C.c_int, C.c_int, vp, C.c_double, C.c_double]
        for name in EXPORTED:
            if name != "sdm_last_error":
                getattr(L, name).restype = C.c_int
        _lib = L
        return L


def _ptr(a):
    return None if a is None else a.ctypes.data


class LangevinParams(C.Structure):
    """``sdm_langevin_params``: step size (ps), friction (1/ps), temperature (K), seed."""
    _fields_ = [("step_size", C.c_double), ("friction", C.c_double), ("temperature", C.c_double),
                ("seed", C.c_ulonglong)]


class RestraintDesc(C.Structure):
    """``sdm_restraints`` (group-1 restraints of the reference's SDMUtils)."""
    _fields_ = [
        ("num_lig", C.c_int), ("num_rcpt", C.c_int),
        ("lig_particles", C.POINTER(C.c_int)), ("rcpt_particles", C.POINTER(C.c_int)),
        ("lig_weights", C.POINTER(C.c_double)), ("rcpt_weights", C.POINTER(C.c_double)),
        ("kfcm", C.c_double), ("tolcm", C.c_double), ("offset", C.c_double * 3),
        ("use_angles", C.c_int), ("rcpt_ref", C.c_int * 3), ("lig_ref", C.c_int * 3),
        ("kf_angle", C.c_double), ("angle_center", C.c_double), ("angle_tol", C.c_double),
        ("kf_dihedral1", C.c_double), ("dihedral1_center", C.c_double), ("dihedral1_tol", C.c_double),
        ("kf_dihedral2", C.c_double), ("dihedral2_center", C.c_double), ("dihedral2_tol", C.c_double),
        ("use_alignment", C.c_int), ("liga_ref", C.c_int * 3), ("ligb_ref", C.c_int * 3),
        ("kf_displ", C.c_double), ("k_theta", C.c_double), ("k_psi", C.c_double),
        ("align_offset", C.c_double * 3),
    ]


def restraint_desc(rs, keep):
    """RestraintDesc of a systems.Restraints (arrays appended to `keep`)."""
    d = RestraintDesc()
    lig = np.ascontiguousarray(np.asarray(rs.lig_particles, np.int32))
    rcpt = np.ascontiguousarray(np.asarray(rs.rcpt_particles, np.int32))
    keep += [lig, rcpt]
    d.num_lig, d.num_rcpt = int(lig.size), int(rcpt.size)
    d.lig_particles = lig.ctypes.data_as(C.POINTER(C.c_int)) if lig.size else None
    d.rcpt_particles = rcpt.ctypes.data_as(C.POINTER(C.c_int)) if rcpt.size else None
    for name, arr in (("lig_weights", rs.lig_weights), ("rcpt_weights", rs.rcpt_weights)):
        if arr is not None:
            w = np.ascontiguousarray(np.asarray(arr, np.float64))
            keep.append(w)
            setattr(d, name, w.ctypes.data_as(C.POINTER(C.c_double)))
    for f in ("kfcm", "tolcm", "kf_angle", "angle_center", "angle_tol", "kf_dihedral1", "dihedral1_center",
              "dihedral1_tol", "kf_dihedral2", "dihedral2_center", "dihedral2_tol", "kf_displ", "k_theta", "k_psi"):
        setattr(d, f, float(getattr(rs, f)))
    d.offset[:] = [float(v) for v in rs.offset]
    d.align_offset[:] = [float(v) for v in rs.align_offset]
    d.use_angles, d.use_alignment = int(bool(rs.use_angles)), int(bool(rs.use_alignment))
    for f in ("rcpt_ref", "lig_ref", "liga_ref", "ligb_ref"):
        getattr(d, f)[:] = [int(v) for v in getattr(rs, f)]
    return d


def system_descs(systems, keep):
    """sdm_system_desc array of systems; the arrays it points to are appended
    to `keep` (they must outlive the array)."""
    descs = (SystemDesc * len(systems))()
    for k, s in enumerate(systems):
        q = np.ascontiguousarray(s.charge, np.float64)
        sg = np.ascontiguousarray(s.sigma, np.float64)
        ep = np.ascontiguousarray(s.epsilon, np.float64)
        ex = np.ascontiguousarray(np.asarray(s.exclusions, np.int32).reshape(-1))
        dd = np.ascontiguousarray(np.asarray(s.displacement, np.float64).reshape(-1))
        keep += [q, sg, ep, ex, dd]
        d = descs[k]
        d.num_particles = int(q.shape[0])
        d.charge = q.ctypes.data_as(C.POINTER(C.c_double))
        d.sigma = sg.ctypes.data_as(C.POINTER(C.c_double))
        d.epsilon = ep.ctypes.data_as(C.POINTER(C.c_double))
        d.num_exclusions = int(ex.shape[0] // 2)
        d.exclusions = ex.ctypes.data_as(C.POINTER(C.c_int)) if ex.size else None
        d.displacement = dd.ctypes.data_as(C.POINTER(C.c_double))
        d.box[:] = [float(v) for v in s.box]
        d.cutoff = float(s.cutoff)
        d.reaction_field_dielectric = float(s.eps_rf)
        d.num_replicas = int(s.positions.shape[0]) if getattr(s, "positions", None) is not None else 1
        if getattr(s, "nonbonded_method", "rf") == "pme":
            d.nonbonded_method = NB_PME
            d.ewald_tolerance = float(getattr(s, "ewald_tolerance", 5e-4))
            g = getattr(s, "pme_grid", None)
            if g is not None:
                d.pme_grid[:] = [int(v) for v in g]
        xp = getattr(s, "exceptions", None)
        if xp is not None and len(xp):
            xpi = np.ascontiguousarray(np.asarray(xp, np.int32).reshape(-1))
            xpp = np.ascontiguousarray(np.asarray(s.exception_params, np.float64).reshape(-1))
            if xpp.size != 3 * (xpi.size // 2):
                raise ValueError("exception_params needs (charge product, sigma, epsilon) per pair")
            keep += [xpi, xpp]
            d.num_exceptions = int(xpi.size // 2)
            d.exception_pairs = xpi.ctypes.data_as(C.POINTER(C.c_int))
            d.exception_params = xpp.ctypes.data_as(C.POINTER(C.c_double))
    return descs


class Handle:
    """Owning wrapper of one ``sdm_handle``.

    ``systems`` is a list of :class:`openmm_sdm_plugin_gb300.systems.SDMSystem`
    (or duck-typed objects with the same fields).
    """

    def __init__(self, systems, device: int = 0):
        self.lib = load_library()
        self.systems = list(systems)
        self._keep = []
        descs = system_descs(self.systems, self._keep)
        h = C.c_void_p()
        st = self.lib.sdm_create(descs, len(self.systems), int(device), C.byref(h))
        if st != SDM_OK:
            raise SdmError(st, self.lib.sdm_last_error(None).decode())
        self.h = h
        n = C.c_int(0)
        self.lib.sdm_num_replicas(self.h, C.byref(n))
        self.nrep = n.value
        self.rep_sys = []
        self.rep_n = []
        for k, s in enumerate(self.systems):
            r = int(s.positions.shape[0]) if getattr(s, "positions", None) is not None else 1
            self.rep_sys += [k] * r
            self.rep_n += [int(s.charge.shape[0])] * r
        self.total_particles = int(sum(self.rep_n))
        for k, s in enumerate(self.systems):
            if getattr(s, "restraints", None) is not None:
                self.set_restraints(k, s.restraints)

    # -- group-1 restraints ------------------------------------------------
    def set_restraints(self, system: int, rs):
        """Restraints (systems.Restraints or None) of one system."""
        keep = []
        d = restraint_desc(rs, keep) if rs is not None else None
        self._check(self.lib.sdm_set_restraints(self.h, int(system), C.byref(d) if d is not None else None))

    def set_restraint_control(self, replica: int, value: float):
        self._check(self.lib.sdm_set_restraint_control(self.h, int(replica), float(value)))

    def set_rigid_waters(self, system: int, waters, d_oh: float = 0.0, d_hh: float = 0.0):
        """Rigid (O, H, H) waters of one system in the Langevin step; waters (W, 3) or None."""
        w = np.ascontiguousarray(np.asarray(waters if waters is not None else [], np.int32).reshape(-1))
        self._check(self.lib.sdm_set_rigid_waters(self.h, int(system), int(w.size // 3),
                                                  w.ctypes.data if w.size else None, float(d_oh), float(d_hh)))

    def restraint_energies(self):
        out = np.zeros(self.nrep)
        self._check(self.lib.sdm_get_restraint_energies(self.h, out.ctypes.data))
        return out

    # -- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.sdm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != SDM_OK:
            raise SdmError(st, self.lib.sdm_last_error(self.h).decode())

    # -- configuration ----------------------------------------------------
    def set_params(self, replica: int, params):
        p = np.ascontiguousarray(np.asarray(params, np.float64).reshape(-1))
        if p.size != NPARAMS:
            raise ValueError(f"need {NPARAMS} parameters")
        self._check(self.lib.sdm_set_params(self.h, int(replica), p.ctypes.data))

    def set_displacement(self, system: int, d):
        dd = np.ascontiguousarray(np.asarray(d, np.float64).reshape(-1))
        self._check(self.lib.sdm_set_displacement(self.h, int(system), dd.ctypes.data))

    def set_option(self, opt: int, value: int):
        self._check(self.lib.sdm_set_option(self.h, int(opt), int(value)))

    def get_option(self, opt: int) -> int:
        v = C.c_int(0)
        self._check(self.lib.sdm_get_option(self.h, int(opt), C.byref(v)))
        return v.value

    def grid(self, system: int = 0):
        M = (C.c_int * 3)()
        self._check(self.lib.sdm_get_grid(self.h, int(system), M))
        return np.array(list(M), np.int32)

    # -- evaluation -------------------------------------------------------
    def set_particle_params(self, system: int, index, charge, sigma, epsilon):
        idx = np.ascontiguousarray(np.asarray(index, np.int32).reshape(-1))
        q = np.ascontiguousarray(np.asarray(charge, np.float64).reshape(-1))
        sg = np.ascontiguousarray(np.asarray(sigma, np.float64).reshape(-1))
        ep = np.ascontiguousarray(np.asarray(epsilon, np.float64).reshape(-1))
        self._check(self.lib.sdm_set_particle_params(self.h, int(system), int(idx.size), idx.ctypes.data,
                                                     q.ctypes.data, sg.ctypes.data, ep.ctypes.data))

    def num_perturbed(self) -> int:
        """(replica, displaced particle) entries of the adjoint output, as the
        library counts them."""
        v = C.c_int(0)
        self._check(self.lib.sdm_get_num_perturbed(self.h, C.byref(v)))
        return v.value

    def adjoint(self, n_displaced=None):
        """Adjoint sums of the last evaluation: (sum over replicas of nD, 2 states, 3).
        The output is sized from the library's own displaced-particle count;
        n_displaced, when given, must equal it."""
        total = self.num_perturbed()
        if n_displaced is not None and int(n_displaced) != total:
            raise ValueError(f"the replicas hold {total} displaced particles, not {int(n_displaced)}")
        out = np.zeros(6 * total)
        self._check(self.lib.sdm_adjoint(self.h, out.ctypes.data))
        return out.reshape(-1, 2, 3)

    def adjoint_device(self, out_ptr: int, stream: int = 0):
        """sdm_adjoint_device: the sums into a device buffer of 6 * num_perturbed()
        doubles, asynchronous on ``stream``."""
        self._check(self.lib.sdm_adjoint_device(self.h, C.c_void_p(out_ptr), _stream(stream)))

    def backward_device(self, grad_u: int, results: int, forces: int = 0, forces1: int = 0, adjoint: int = 0,
                        eps_displaced: int = 0, bias_params: int = 0, grad_x: int = 0, grad_d: int = 0,
                        grad_p: int = 0, grad_bias: int = 0, stream: int = 0):
        """sdm_backward_device: gradients of the replicas' potentials from
        dL/dU (device pointers; 0 = NULL), asynchronous on ``stream``."""
        v = lambda p: C.c_void_p(p) if p else None
        self._check(self.lib.sdm_backward_device(self.h, v(grad_u), v(results), v(forces), v(forces1), v(adjoint),
                                                 v(eps_displaced), v(bias_params), v(grad_x), v(grad_d),
                                                 v(grad_p), v(grad_bias), _stream(stream)))

    def set_langevin(self, step_size: float, friction: float, temperature: float, seed: int = 0,
                     step: int = 0):
        p = LangevinParams(float(step_size), float(friction), float(temperature), int(seed))
        self._check(self.lib.sdm_set_langevin(self.h, C.byref(p), int(step)))

    def langevin_step(self, x_ptr: int, v_ptr: int, inv_mass_ptr: int, res_ptr: int, nsteps: int = 1,
                      f_extra_ptr: int = 0, stream: int = 0):
        """nsteps fused Langevin steps on device buffers (asynchronous on ``stream``)."""
        self._check(self.lib.sdm_langevin_step(self.h, C.c_void_p(x_ptr), C.c_void_p(v_ptr),
                                               C.c_void_p(inv_mass_ptr),
                                               C.c_void_p(f_extra_ptr) if f_extra_ptr else None,
                                               C.c_void_p(res_ptr), int(nsteps),
                                               _stream(stream)))

    def evaluate(self, x, forces: bool = True):
        """Host evaluation of all replicas. x: (total_particles, 3) float64."""
        x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1))
        if x.size != 3 * self.total_particles:
            raise ValueError("coordinate array has the wrong size")
        res = np.zeros((self.nrep, NRESULTS))
        f = np.zeros(3 * self.total_particles) if forces else None
        self._check(self.lib.sdm_evaluate(self.h, x.ctypes.data, res.ctypes.data, _ptr(f)))
        return res, (f.reshape(-1, 3) if forces else None)

    def evaluate_host_ptrs(self, x_ptr: int, res_ptr: int, f_ptr: int = 0):
        """sdm_evaluate on caller-owned host buffers given by address (page-locked
        coordinates are read in place by the kernels)."""
        self._check(self.lib.sdm_evaluate(self.h, C.c_void_p(x_ptr), C.c_void_p(res_ptr) if res_ptr else None,
                                          C.c_void_p(f_ptr) if f_ptr else None))

    def evaluate_device(self, x_ptr: int, res_ptr: int, f_ptr: int = 0, stream: int = 0):
        self._check(self.lib.sdm_evaluate_device(self.h, C.c_void_p(x_ptr), C.c_void_p(res_ptr),
                                                 C.c_void_p(f_ptr) if f_ptr else None,
                                                 _stream(stream)))

    def state_forces(self):
        F0 = np.zeros(3 * self.total_particles)
        F1 = np.zeros(3 * self.total_particles)
        self._check(self.lib.sdm_get_state_forces(self.h, F0.ctypes.data, F1.ctypes.data, 0))
        return F0.reshape(-1, 3), F1.reshape(-1, 3)

    def state_forces_device(self, F0_ptr: int = 0, F1_ptr: int = 0, stream: int = 0):
        """sdm_get_state_forces_device: F0 and/or F1 of the last evaluation into
        device buffers, asynchronous on ``stream``."""
        self._check(self.lib.sdm_get_state_forces_device(self.h, C.c_void_p(F0_ptr) if F0_ptr else None,
                                                         C.c_void_p(F1_ptr) if F1_ptr else None,
                                                         _stream(stream)))

    def check_status(self) -> int:
        v = C.c_int(0)
        self._check(self.lib.sdm_check_status(self.h, C.byref(v)))
        return v.value

    def kernel_times(self):
        names = (C.c_char_p * 16)()
        ms = (C.c_float * 16)()
        n = C.c_int(16)
        self._check(self.lib.sdm_get_kernel_times(self.h, names, ms, C.byref(n)))
        return {names[k].decode(): float(ms[k]) for k in range(n.value)}

    def autotune(self, x_ptr: int, cache_path=None):
        """sdm_autotune_cached on device coordinates: dict of the chosen
        stage_chunk, ctas_per_sm, split, list_group, overlap, the median ms
        and from_cache."""
        r = TuneResult()
        self._check(self.lib.sdm_autotune_cached(self.h, C.c_void_p(x_ptr),
                                                 cache_path.encode() if cache_path else None, C.byref(r)))
        return dict(stage_chunk=r.stage_chunk, ctas_per_sm=r.ctas_per_sm, split=r.split, ms=r.ms,
                    from_cache=bool(r.from_cache), list_group=r.list_group, overlap=r.overlap)

    def count_pairs(self, x):
        x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1))
        c = np.zeros(2 * self.nrep, np.int64)
        self._check(self.lib.sdm_count_pairs(self.h, x.ctypes.data, c.ctypes.data))
        return c.reshape(-1, 2)

    def export_lists(self, replica: int, x, cap_per_cluster: int = 2048):
        x = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1))
        n = self.rep_n[replica]
        M = self.grid(self.rep_sys[replica])
        cap_slots = n + 8 * int(M[0] * M[1]) + 16
        capcl = cap_slots // 8 + 1
        perm = np.zeros(cap_slots, np.int32)
        cnt = np.zeros(capcl, np.int32)
        es = np.zeros(capcl * cap_per_cluster, np.int32)
        em = np.zeros(capcl * cap_per_cluster, np.uint8)
        ncl = C.c_int(0)
        self._check(self.lib.sdm_export_lists(self.h, int(replica), x.ctypes.data, cap_slots, capcl,
                                              cap_per_cluster, perm.ctypes.data, C.byref(ncl),
                                              cnt.ctypes.data, es.ctypes.data, em.ctypes.data))
        k = ncl.value
        return dict(ncl=k, perm=perm[:8 * k], cnt=cnt[:k], slot=es.reshape(capcl, -1)[:k],
                    mask=em.reshape(capcl, -1)[:k])


def evaluate_noalloc(n, x_ptr, q_ptr, sig_ptr, eps_ptr, eoff_ptr, eidx_ptr, d_ptr, box, cutoff,
                     eps_rf, params, res_ptr, f_ptr=0, stream=0):
    """Allocation-free evaluation of one system (device pointers, see
    sdm_evaluate_noalloc in include/sdm_capi.h)."""
    L = load_library()
    b = np.ascontiguousarray(np.asarray(box, np.float64).reshape(3))
    p = np.ascontiguousarray(np.asarray(params, np.float64).reshape(-1))
    st = L.sdm_evaluate_noalloc(int(n), C.c_void_p(x_ptr), C.c_void_p(q_ptr), C.c_void_p(sig_ptr),
                                C.c_void_p(eps_ptr), C.c_void_p(eoff_ptr), C.c_void_p(eidx_ptr),
                                C.c_void_p(d_ptr) if d_ptr else None, b.ctypes.data,
                                float(cutoff), float(eps_rf), p.ctypes.data, C.c_void_p(res_ptr),
                                C.c_void_p(f_ptr) if f_ptr else None,
                                _stream(stream))
    if st != SDM_OK:
        raise SdmError(st, L.sdm_last_error(None).decode())


def tune_key(systems, num_sms: int) -> str:
    """The autotuner's cache key of a workload (sdm_tune_key; no device needed)."""
    L = load_library()
    keep = []
    descs = system_descs(list(systems), keep)
    buf = C.create_string_buffer(256)
    st = L.sdm_tune_key(descs, len(systems), int(num_sms), buf, 256)
    if st != SDM_OK:
        raise SdmError(st, "sdm_tune_key failed")
    return buf.value.decode()
