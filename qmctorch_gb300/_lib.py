"""Build and load ``libqmc_gb300.so`` (the sm_103a kernels) and describe its C
ABI (``include/qmc_gb300.h``) with ctypes.

The library is built in-tree (``qmctorch_gb300/lib``) with nvcc, one
translation unit per process, and loaded with ``ctypes.CDLL``. There is no
CPU fallback: every compute entry point of the package goes through this
library, and :func:`lib` raises when it cannot be loaded.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIBPATH = os.path.join(LIBDIR, "libqmc_gb300.so")
BUILD = os.path.join(ROOT, "_build")
INCLUDE = os.path.join(ROOT, "include")

SOURCES = ["qmc_wf_kernels.cu", "qmc_staged.cu", "qmc_metropolis.cu", "qmc_capi_common.cu",
           "qmc_probe.cu", "qmc_adjoint.cu", "qmc_drift.cu", "qmc_sweep.cu", "qmc_reduce.cu",
           "qmc_mo_tc.cu", "qmc_scf.cpp"]
# translation units compiled more than once, with defines: (source, object, flags)
INSTANCES = [("qmc_metropolis_inst.cu", "qmc_metropolis_%s_%d" % (r, jc),
              ["-DQMC_INST_R=%s" % r, "-DQMC_INST_JC=%d" % jc])
             for r in ("float", "double") for jc in (8, 16, 24)]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE]


def _nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build qmc_gb300")
    return path


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    """Compile every translation unit for sm_103a and link the shared library."""
    if not force and os.path.exists(LIBPATH) and os.path.getmtime(LIBPATH) >= _deps_mtime():
        return LIBPATH
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(unit):
        src, name, flags = unit
        obj = os.path.join(BUILD, name + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    units = [(src, os.path.splitext(src)[0], []) for src in SOURCES] + INSTANCES
    # longest first: the Metropolis and sweep units set the wall time
    units.sort(key=lambda u: ("inst" not in u[0], "sweep" not in u[0]))
    with ThreadPoolExecutor(max_workers=min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIBPATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-Xlinker",
                           "-rpath,/usr/local/cuda/lib64", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIBPATH)
    return LIBPATH


# ----------------------------------------------------------------------------
# C structures (must match include/qmc_gb300.h)
# ----------------------------------------------------------------------------
c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_void_p = ctypes.c_void_p


class WfDesc(ctypes.Structure):
    _fields_ = [
        ("nelec", c_int32), ("nup", c_int32), ("ndown", c_int32), ("natom", c_int32),
        ("nao", c_int32), ("nmo", c_int32), ("nmo_used", c_int32), ("ngroup", c_int32),
        ("ngprim", c_int32), ("nweight", c_int32), ("contract", c_int32),
        ("use_jastrow", c_int32), ("precision", c_int32),
        ("atom_coords", c_void_p), ("atom_charge", c_void_p), ("group_atom", c_void_p),
        ("group_prim", c_void_p), ("group_ao", c_void_p), ("gprim_entry", c_void_p),
        ("bas_exp", c_void_p), ("ao_k", c_void_p), ("ao_wofs", c_void_p), ("weight_entry", c_void_p),
        ("ao_wd", c_void_p),
        ("ao_wv", c_void_p), ("mo_scf", c_void_p), ("mo_modifier", c_void_p),
        ("jastrow_w", c_void_p),
        ("det_mode", c_int32), ("ncfg", c_int32), ("max_orb", c_int32 * 2),
        ("ndet", c_int32 * 2), ("det_table", c_void_p * 2), ("cfg_det", c_void_p * 2),
        ("ci_weight", c_void_p), ("e_nuc", ctypes.c_double),
        ("use_jastrow_en", c_int32), ("jastrow_en_w", c_void_p), ("jastrow_en_atoms", c_void_p),
        ("radial_type", c_int32), ("ao_kr", c_void_p),
    ]


class GtoBasis(ctypes.Structure):
    _fields_ = [("nao", c_int32), ("nprim", c_int32), ("prim_ao", c_void_p),
                ("prim_center", c_void_p), ("prim_exp", c_void_p), ("prim_coef", c_void_p),
                ("prim_k", c_void_p)]


class MetropolisArgs(ctypes.Structure):
    _fields_ = [
        ("pos", c_void_p), ("nwalkers", c_int64), ("nstep", c_int32), ("ntherm", c_int32),
        ("ndecor", c_int32), ("move_type", c_int32), ("proba", c_int32),
        ("step_size", ctypes.c_double), ("seed", ctypes.c_uint64),
        ("step_offset", ctypes.c_uint64), ("samples", c_void_p), ("nsnap", c_int64),
        ("accepted", c_void_p), ("psi_out", c_void_p), ("proposals", c_void_p),
        ("uniforms", c_void_p), ("electron_index", c_void_p),
    ]


class DriftArgs(ctypes.Structure):
    _fields_ = [
        ("pos", c_void_p), ("nwalkers", c_int64), ("nstep", c_int32), ("ntherm", c_int32),
        ("ndecor", c_int32), ("step_size", ctypes.c_double), ("seed", ctypes.c_uint64),
        ("step_offset", ctypes.c_uint64), ("samples", c_void_p), ("nsnap", c_int64),
        ("accepted", c_void_p), ("electron_index", c_void_p), ("normals", c_void_p),
        ("uniforms", c_void_p),
    ]


class HmcArgs(ctypes.Structure):
    _fields_ = [
        ("pos", c_void_p), ("nwalkers", c_int64), ("nstep", c_int32), ("ntherm", c_int32),
        ("ndecor", c_int32), ("traj_length", c_int32), ("step_size", ctypes.c_double),
        ("seed", ctypes.c_uint64), ("step_offset", ctypes.c_uint64), ("samples", c_void_p),
        ("nsnap", c_int64), ("accepted", c_void_p), ("momenta", c_void_p),
        ("uniforms", c_void_p),
    ]


# every symbol include/qmc_gb300.h declares: name -> (restype, argtypes)
_P = ctypes.POINTER
SIGNATURES = {
    "qmc_version": (ctypes.c_char_p, []),
    "qmc_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "qmc_scratch_bytes": (c_int64, [_P(WfDesc), c_int64, c_int32]),
    "qmc_metropolis_scratch_bytes": (c_int64, [_P(WfDesc), c_int64]),
    "qmc_metropolis_plan": (ctypes.c_int, [_P(WfDesc), c_int64, _P(c_int32)]),
    "qmc_wf_psi": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                  c_void_p]),
    "qmc_wf_psi_static": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p]),
    "qmc_wf_local_energy": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p,
                                           c_void_p, c_void_p, c_int64, c_void_p]),
    "qmc_ao_eval": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_int32, c_void_p, c_void_p,
                                   c_void_p, c_void_p]),
    "qmc_mo_eval": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p]),
    "qmc_mo_eval_tc": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p]),
    "qmc_mo_eval_tc_status": (ctypes.c_int, [c_void_p]),
    "qmc_scf_one_electron": (ctypes.c_int, [_P(GtoBasis), c_int32, c_void_p, c_void_p, c_void_p,
                                            c_void_p, c_void_p]),
    "qmc_scf_eri": (ctypes.c_int, [_P(GtoBasis), c_void_p]),
    "qmc_jastrow_en": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p,
                                      c_void_p, c_int32, c_void_p]),
    "qmc_set_wait_limit_ns": (ctypes.c_uint64, [ctypes.c_uint64]),
    "qmc_jastrow_ee": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p,
                                      c_void_p, c_int32, c_void_p]),
    "qmc_slater": (ctypes.c_int, [_P(WfDesc), c_void_p, c_void_p, c_int32, c_int64, c_void_p,
                                  c_void_p, c_void_p, c_int64, c_void_p]),
    "qmc_potentials": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p,
                                      c_void_p]),
    "qmc_adjoint_scratch_bytes": (c_int64, [_P(WfDesc), c_int64]),
    "qmc_wf_psi_adjoint": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p, c_void_p,
                                          c_int32, c_void_p, c_void_p, c_int32, c_void_p,
                                          c_void_p, c_void_p, c_int64, c_void_p]),
    "qmc_eloc_adjoint_scratch_bytes": (c_int64, [_P(WfDesc), c_int64]),
    "qmc_wf_local_energy_adjoint": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_void_p,
                                                   c_void_p, c_int32, c_void_p, c_void_p, c_int32,
                                                   c_void_p, c_void_p, c_void_p, c_int64,
                                                   c_void_p]),
    "qmc_grad_scratch_bytes": (c_int64, [_P(WfDesc), c_int64]),
    "qmc_wf_gradients": (ctypes.c_int, [_P(WfDesc), c_void_p, c_int64, c_int32, c_void_p,
                                        c_void_p, c_int64, c_void_p]),
    "qmc_probe_fma": (ctypes.c_int, [c_int32, c_int32, c_int64, c_void_p, c_void_p]),
    "qmc_probe_exp64": (ctypes.c_int, [c_void_p, c_int64, c_void_p, c_void_p]),
    "qmc_drift_scratch_bytes": (c_int64, [_P(WfDesc), c_int64]),
    "qmc_drift_run": (ctypes.c_int, [_P(WfDesc), _P(DriftArgs), c_void_p, c_int64, c_void_p]),
    "qmc_hmc_scratch_bytes": (c_int64, [_P(WfDesc), c_int64]),
    "qmc_hmc_run": (ctypes.c_int, [_P(WfDesc), _P(HmcArgs), c_void_p, c_int64, c_void_p]),
    "qmc_metropolis_run": (ctypes.c_int, [_P(WfDesc), _P(MetropolisArgs), c_void_p, c_int64,
                                          c_void_p]),
    "qmc_metropolis_run_batch": (ctypes.c_int, [_P(WfDesc), _P(MetropolisArgs), _P(c_void_p),
                                                _P(c_int64), c_int32, c_void_p]),
    "qmc_reduce_scratch_bytes": (c_int64, [c_int64]),
    "qmc_reduce_stats": (ctypes.c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_int64,
                                        c_void_p]),
}

_LIB = None


def lib():
    """Load the shared library (building it first if it is missing)."""
    global _LIB
    if _LIB is None:
        build()  # no-op while the library is newer than its sources
        import torch  # noqa: F401  (loads the CUDA runtime the library links against)
        handle = ctypes.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


class QMCError(RuntimeError):
    pass


def check(status, what):
    if status != 0:
        msg = lib().qmc_status_string(status).decode()
        raise QMCError("%s failed: %s (status %d)" % (what, msg, status))
