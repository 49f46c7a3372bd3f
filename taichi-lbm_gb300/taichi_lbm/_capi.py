"""ctypes binding of liblbm_gb300.so (declarations in include/lbm_gb300.h).

The library is the only compute path of this package: importing it without
the built library, or using it without a CUDA device, raises immediately.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblbm_gb300.so")

# enums (lbm_gb300.h)
LBM_OK = 0
BGK, TRT, MRT = 0, 1, 2
NEWTONIAN, POWERLAW = 0, 1
STORE_F32, STORE_F16S, STORE_BF16S, STORE_I16S = 0, 1, 2, 3
EOS_SC, EOS_VDW, EOS_RK, EOS_PR, EOS_CS = 0, 1, 2, 3, 4
BC_FLUID, BC_VELOCITY_BB, BC_VELOCITY_EQ, BC_VELOCITY_NEEM = 0, 1, 2, 3
BC_PRESSURE_ABC, BC_PRESSURE_NEEM, BC_OPEN_NEUMANN, BC_OPEN_CONV1 = 4, 5, 6, 7
BC_OPEN_CONV2, BC_OPEN_EXTRAP, BC_PERIODIC, BC_INSIDE, BC_BOUNCEBACK = 8, 9, 10, 11, 12
MAX_BC, MAX_PROG, PROG_LEN = 16, 64, 4
CODE_ACTIVE, CODE_SAVE, CODE_PROG_SHIFT = 0x100, 0x200, 10

_fp = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p


class LbmLattice(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("pitch", ctypes.c_int32),
                ("psi_pitch", ctypes.c_int32)] + [
        (n, _vp) for n in ("f", "f2", "rho", "total_rho", "pressure", "total_pressure",
                           "shear_rate", "temperature", "vel", "body_force", "sc_force", "psi",
                           "mask", "links")] + [("gravity", ctypes.c_float * 2)]


class LbmIBNodes(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [(n, _vp) for n in ("pos", "vel", "vel_desired", "force", "force_temp")]


class LbmCollision(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int32), ("fluid_model", ctypes.c_int32),
                ("nu", ctypes.c_float), ("nu_bulk", ctypes.c_float), ("magic", ctypes.c_float),
                ("tau_min", ctypes.c_float), ("tau_max", ctypes.c_float),
                ("pl_m", ctypes.c_float), ("pl_n", ctypes.c_float),
                ("tau", _vp), ("tau_sym", _vp), ("tau_antisym", _vp), ("diag", _vp),
                ("m_inverse", ctypes.c_float * 81)]


class LbmEos(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("a", ctypes.c_float), ("b", ctypes.c_float),
                ("R", ctypes.c_float), ("G", ctypes.c_float), ("rho0", ctypes.c_float),
                ("omega", ctypes.c_float), ("T_cr", ctypes.c_float)]


MC_MAX = 4


class LbmMCLattice(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("pitch", ctypes.c_int32),
                ("psi_pitch", ctypes.c_int32), ("nc", ctypes.c_int32)] + [
        (n, _vp) for n in ("f", "f2", "rho", "total_rho", "pressure", "total_pressure", "temperature",
                           "vel", "body_force", "sc_force", "psi")] + [("gravity", ctypes.c_float * 2)]


class LbmMCShanChen(ctypes.Structure):
    _fields_ = [("g_coh", (ctypes.c_float * MC_MAX) * MC_MAX), ("g_adh", ctypes.c_float * MC_MAX),
                ("eos", LbmEos * MC_MAX), ("fluid", _vp)]


class LbmBoundary(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("direction", ctypes.c_int32),
                ("rho_value", ctypes.c_float), ("velocity", ctypes.c_float * 2),
                ("velocity_per_node", _vp), ("g_coh", ctypes.c_float), ("eos", LbmEos)]


class LbmPlanDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("pitch", ctypes.c_int32),
                ("model", ctypes.c_int32), ("fluid_model", ctypes.c_int32),
                ("storage", ctypes.c_int32), ("nodes_per_thread", ctypes.c_int32),
                ("tau", ctypes.c_float), ("tau_antisym", ctypes.c_float), ("magic", ctypes.c_float),
                ("tau_min", ctypes.c_float), ("tau_max", ctypes.c_float),
                ("pl_m", ctypes.c_float), ("pl_n", ctypes.c_float),
                ("mrt_s", ctypes.c_float * 9), ("gravity", ctypes.c_float * 2),
                ("nbc", ctypes.c_int32), ("bc", LbmBoundary * MAX_BC),
                ("nprog", ctypes.c_int32), ("prog", (ctypes.c_int8 * PROG_LEN) * MAX_PROG),
                ("pipeline", ctypes.c_int32), ("tune", ctypes.c_int32),
                ("sc", ctypes.c_int32), ("g_coh", ctypes.c_float), ("sc_T", ctypes.c_float),
                ("eos", LbmEos), ("rho_ref", ctypes.c_float), ("fixed_exp", ctypes.c_int32),
                ("wait_cycles", ctypes.c_int64), ("aa", ctypes.c_int32)]


# fixed-point storage step 2^-fixed_exp (range 2^(15 - fixed_exp))
FIXED_EXP_DEFAULT, FIXED_EXP_MIN, FIXED_EXP_MAX = 19, 12, 22
# sticky bits of a plan's device status word
STATUS_TIMEOUT, STATUS_SATURATED, STATUS_NONFINITE = 1, 2, 4
# open psi boundary kinds (lbm_psi_open)
PSI_OPEN_NEUMANN, PSI_OPEN_CONV1, PSI_OPEN_CONV2, PSI_OPEN_EXTRAP = 0, 1, 2, 3

PIPE_DIRECT, PIPE_ASYNC, PIPE_PREFETCH = 0, 1, 2
ASYNC_TUNINGS = 4


class LbmPlanBuffers(ctypes.Structure):
    _fields_ = [(n, _vp) for n in ("fa", "fb", "mom_a", "mom_b", "code", "seg_flags", "bc_vel",
                                   "tau", "status", "special")] + [("nspecial", ctypes.c_int32),
                                                           ("special_stream", ctypes.c_int32),
                                                           ("plain", _vp), ("nplain", ctypes.c_int32),
                                                           ("lane_mask", _vp), ("lanes", _vp),
                                                           ("nlanes", ctypes.c_int32),
                                                           ("aa_sites", _vp), ("aa_nsites", ctypes.c_int32),
                                                           ("aa_vals", _vp)]


class LbmError(RuntimeError):
    """A liblbm_gb300 call returned an error status."""


_lib = None

_SIGS = {
    "lbm_abi_version": ([], ctypes.c_int),
    "lbm_last_error": ([ctypes.c_char_p, ctypes.c_int64], ctypes.c_int),
    "lbm_neighbor_classify": ([ctypes.POINTER(LbmLattice), _vp], ctypes.c_int),
    "lbm_init_feq": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_density": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_pressure": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, ctypes.c_int32,
                      ctypes.c_float, _vp], ctypes.c_int),
    "lbm_force_density": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_velocity": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_ibm_interpolate": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmIBNodes), _vp], ctypes.c_int),
    "lbm_ibm_spread": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmIBNodes), _vp], ctypes.c_int),
    "lbm_collision_init_tau": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmCollision), _vp,
                                ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_collision_shear_rate": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmCollision), _vp,
                                  ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_collision_relaxation_time": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmCollision),
                                       _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_collision_apply": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmCollision), _vp,
                             ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_sc_update_psi": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmEos), _vp,
                           ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_sc_force": ([ctypes.POINTER(LbmLattice), ctypes.c_float, _vp, ctypes.c_int64, _vp],
                     ctypes.c_int),
    "lbm_psi_periodic": ([ctypes.POINTER(LbmLattice), ctypes.c_int32, _vp], ctypes.c_int),
    "lbm_psi_fixed": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, ctypes.c_float, _vp],
                      ctypes.c_int),
    "lbm_psi_open": ([ctypes.POINTER(LbmLattice), _vp, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, _vp],
                     ctypes.c_int),
    "lbm_mc_init_feq": ([ctypes.POINTER(LbmMCLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_density": ([ctypes.POINTER(LbmMCLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_pressure2": ([ctypes.POINTER(LbmMCLattice), ctypes.POINTER(LbmMCShanChen), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_update_psi": ([ctypes.POINTER(LbmMCLattice), ctypes.POINTER(LbmMCShanChen), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_psi_periodic": ([ctypes.POINTER(LbmMCLattice), ctypes.c_int32, _vp], ctypes.c_int),
    "lbm_mc_sc_force": ([ctypes.POINTER(LbmMCLattice), ctypes.POINTER(LbmMCShanChen), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_force_density": ([ctypes.POINTER(LbmMCLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_velocity": ([ctypes.POINTER(LbmMCLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_bgk_apply": ([ctypes.POINTER(LbmMCLattice), _vp, _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_mc_stream_periodic": ([ctypes.POINTER(LbmMCLattice), _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_boundary_apply": ([ctypes.POINTER(LbmLattice), ctypes.POINTER(LbmBoundary), _vp,
                            ctypes.c_int64, _vp], ctypes.c_int),
    "lbm_plan_create": ([ctypes.POINTER(LbmPlanDesc), ctypes.POINTER(_vp)], ctypes.c_int),
    "lbm_plan_bind": ([_vp, ctypes.POINTER(LbmPlanBuffers)], ctypes.c_int),
    "lbm_plan_run": ([_vp, ctypes.c_int32, _vp], ctypes.c_int),
    "lbm_plan_get_parity": ([_vp, ctypes.POINTER(ctypes.c_int32)], ctypes.c_int),
    "lbm_plan_set_parity": ([_vp, ctypes.c_int32], ctypes.c_int),
    "lbm_plan_stream": ([_vp, _vp, _vp], ctypes.c_int),
    "lbm_plan_import": ([_vp, _vp, _vp], ctypes.c_int),
    "lbm_plan_export": ([_vp, _vp, _vp], ctypes.c_int),
    "lbm_plan_destroy": ([_vp], ctypes.c_int),
    "lbm_plan_momentum_exchange": ([_vp, _vp, ctypes.c_int64, _vp, _vp], ctypes.c_int),
    "lbm_plan_run_monitored": ([_vp, ctypes.c_int32, _vp, ctypes.c_int64, _vp, _vp], ctypes.c_int),
    "lbm_reduce_scratch_doubles": ([], ctypes.c_int64),
    "lbm_plan_reduce_moments_noalloc": ([_vp, _vp, _vp], ctypes.c_int),
    "lbm_plan_reduce_moments": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "lbm_batch_create": ([_vp], ctypes.c_int),
    "lbm_batch_add": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "lbm_batch_remove": ([_vp, ctypes.c_int32], ctypes.c_int),
    "lbm_batch_monitor": ([_vp, ctypes.c_int32, _vp, ctypes.c_int64, _vp, _vp, ctypes.c_int32], ctypes.c_int),
    "lbm_batch_set_graph": ([_vp, ctypes.c_int32], ctypes.c_int),
    "lbm_batch_set_solo": ([_vp, ctypes.c_int64], ctypes.c_int),
    "lbm_batch_set_sc_rows": ([_vp, ctypes.c_int32], ctypes.c_int),
    "lbm_batch_set_lean_form": ([_vp, ctypes.c_int32], ctypes.c_int),
    "lbm_batch_run": ([_vp, ctypes.c_int32, _vp], ctypes.c_int),
    "lbm_batch_info": ([_vp, _vp, _vp, _vp], ctypes.c_int),
    "lbm_batch_destroy": ([_vp], ctypes.c_int),
}

EXPORTED = tuple(_SIGS)


ABI_VERSION = 4


def load():
    """Load the library (no CUDA call is made here)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with taichi-lbm_gb300/build.py "
                          "(or __graft_entry__.build()); there is no non-CUDA fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    if lib.lbm_abi_version() != ABI_VERSION:  # the structs above follow this version of lbm_gb300.h
        raise ImportError(f"{LIB_PATH} has ABI version {lib.lbm_abi_version()}, these bindings {ABI_VERSION}: "
                          "rebuild it")
    _lib = lib
    return lib


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().lbm_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc, what=""):
    if rc != LBM_OK:
        raise LbmError(f"{what}: {last_error()} (status {rc})")
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args), name)
