"""Python host interface over the C-ABI of libimdgpu (include/imdgpu.h).

Names and meaning follow IMD's own routines for this path (itapmd/imd):
calc_forces (src/imd_forces_nbl.c:281), make_nblist (:136), check_nblist
(:2007), deallocate_nblist (:56), estimate_nblist_size (:74),
move_atoms_nve (src/imd_integrate.c:32), reset_cg / cg_step
(src/imd_cg.c:30, :46).  The GPU library is the only implementation: if it
cannot be loaded the constructor raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# IMDGPU_LIB names another build of the library, e.g. the bounds-checked
# libimdgpu_check.so (python -m imd_gb300.build --check)
LIBPATH = os.environ.get("IMDGPU_LIB") or os.path.join(HERE, "libimdgpu.so")

PAIR, EAM2 = 0, 1
QUADRATIC, FOURPOINT, SPLINE = 0, 1, 2
FP64, MIXED = 0, 1
TAB_PAIR, TAB_RHO, TAB_EMBED = 0, 1, 2
WARN_SHORT = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Scalars(C.Structure):
    _fields_ = [("tot_pot_energy", C.c_double), ("virial", C.c_double),
                ("tot_kin_energy", C.c_double), ("fnorm", C.c_double),
                ("f_max2", C.c_double), ("max_atom_force", C.c_double),
                ("nfc", C.c_long), ("nbl_count", C.c_long), ("nb_entries", C.c_long),
                ("have_valid_nbl", C.c_int), ("gdim", C.c_int * 3), ("nghost", C.c_int),
                ("max_cell_atoms", C.c_int), ("short_distance", C.c_int)]


class GlokParams(C.Structure):
    """imdgpu_glok_params: IMD's glok parameters and build options."""
    _fields_ = [("mix", C.c_int), ("adapt", C.c_int), ("glok_ekin_threshold", C.c_double),
                ("glok_fmaxcrit", C.c_double), ("glok_mix", C.c_double),
                ("glok_mixdec", C.c_double), ("glok_incfac", C.c_double),
                ("glok_decfac", C.c_double), ("glok_maxtimestep", C.c_double),
                ("glok_minsteps", C.c_int), ("min_nPxF", C.c_int), ("steps_min", C.c_int),
                ("nactive", C.c_long)]


class GlokState(C.Structure):
    """imdgpu_glok_state: IMD's globals of the glok ensemble."""
    _fields_ = [("timestep", C.c_double), ("mix", C.c_double),
                ("mixforcescalefac", C.c_double), ("PxF", C.c_double), ("pnorm", C.c_double),
                ("glok_start", C.c_int), ("glok_int", C.c_int), ("nPxF", C.c_int)]


class NptParams(C.Structure):
    """imdgpu_npt_params: IMD's npt_iso parameters."""
    _fields_ = [("temperature", C.c_double), ("isq_tau_eta", C.c_double), ("eta", C.c_double),
                ("isq_tau_xi", C.c_double), ("xi", C.c_double), ("pressure_ext", C.c_double),
                ("pressure_end", C.c_double), ("use_curr_pressure", C.c_int),
                ("steps_min", C.c_int), ("steps_max", C.c_int), ("nactive", C.c_long),
                ("cell_size_tolerance", C.c_double)]


class NptState(C.Structure):
    """imdgpu_npt_state: IMD's globals of ensemble npt_iso."""
    _fields_ = [("xi", C.c_double), ("eta", C.c_double), ("pressure", C.c_double),
                ("pressure_ext", C.c_double), ("volume", C.c_double), ("box", C.c_double * 9)]


class NptAxialParams(C.Structure):
    """imdgpu_npt_axial_params: IMD's npt_axial parameters."""
    _d3 = C.c_double * 3
    _fields_ = [("temperature", C.c_double), ("isq_tau_eta", C.c_double), ("eta", C.c_double),
                ("isq_tau_xi", C.c_double), ("xi", _d3), ("pressure_ext", _d3),
                ("pressure_end", _d3), ("relax_dirs", C.c_int * 3),
                ("use_curr_pressure", C.c_int), ("steps_min", C.c_int), ("steps_max", C.c_int),
                ("nactive", C.c_long), ("cell_size_tolerance", C.c_double)]


class NptAxialState(C.Structure):
    """imdgpu_npt_axial_state: IMD's globals of ensemble npt_axial."""
    _d3 = C.c_double * 3
    _fields_ = [("xi", _d3), ("eta", C.c_double), ("stress", _d3), ("pressure_ext", _d3),
                ("vir_axial", _d3), ("volume", C.c_double), ("box", C.c_double * 9)]


class Timing(C.Structure):
    _fields_ = [("ms_total", C.c_double), ("ms_density", C.c_double),
                ("ms_force", C.c_double), ("ms_integrate", C.c_double),
                ("ms_rebuild", C.c_double), ("steps", C.c_int), ("rebuilds", C.c_int),
                ("kernel_launches", C.c_long)]


class IMDGPUError(RuntimeError):
    pass


_lib = None


def lib() -> C.CDLL:
    """Load libimdgpu.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            if os.environ.get("IMDGPU_LIB"):
                raise IMDGPUError("IMDGPU_LIB names a missing library: " + LIBPATH)
            from . import build
            build.build()
        L = C.CDLL(LIBPATH)
        L.imdgpu_last_error.restype = C.c_char_p
        L.imdgpu_version.restype = C.c_char_p
        L.imdgpu_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int]
        vp = C.c_void_p
        L.imdgpu_destroy.argtypes = [vp]
        L.imdgpu_set_precision.argtypes = [vp, C.c_int]
        L.imdgpu_set_exact.argtypes = [vp, C.c_int]
        L.imdgpu_set_deterministic.argtypes = [vp, C.c_int]
        L.imdgpu_format_atoms.argtypes = [vp, C.c_int, _ip, C.c_int, C.c_char_p, C.c_long,
                                          C.POINTER(C.c_long)]
        L.imdgpu_format_fixed.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_long,
                                          C.POINTER(C.c_long)]
        L.imdgpu_set_graphs.argtypes = [vp, C.c_int]
        L.imdgpu_set_table_staging.argtypes = [vp, C.c_int]
        L.imdgpu_get_tile.argtypes = [vp, C.POINTER(C.c_int)]
        L.imdgpu_set_pair_cache.argtypes = [vp, C.c_int]
        L.imdgpu_set_interpolation.argtypes = [vp, C.c_int]
        L.imdgpu_set_table2.argtypes = [vp, C.c_int, C.c_int, C.c_int, _dp]
        L.imdgpu_set_table.argtypes = [vp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp,
                                       _ip, _dp]
        L.imdgpu_read_table.argtypes = [vp, C.c_int, C.c_char_p, C.c_int, C.c_int]
        L.imdgpu_set_box.argtypes = [vp, _dp, _ip, C.c_double, C.c_double]
        L.imdgpu_set_restrictions.argtypes = [vp, _dp]
        L.imdgpu_set_atoms.argtypes = [vp, C.c_int, _ip, _ip, _dp, _dp, _dp]
        L.imdgpu_get_atoms.argtypes = [vp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.imdgpu_get_scalars.argtypes = [vp, C.POINTER(Scalars)]
        L.imdgpu_calc_forces.argtypes = [vp, C.c_int]
        L.imdgpu_make_nblist.argtypes = [vp]
        L.imdgpu_check_nblist.argtypes = [vp]
        L.imdgpu_deallocate_nblist.argtypes = [vp]
        L.imdgpu_estimate_nblist_size.argtypes = [vp, C.POINTER(C.c_long)]
        L.imdgpu_move_atoms_nve.argtypes = [vp, C.c_double]
        L.imdgpu_nve_run.argtypes = [vp, C.c_int, C.c_double, _dp, _dp]
        L.imdgpu_set_cg_params.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double,
                                           C.c_double, C.c_double, C.c_int, C.c_int]
        L.imdgpu_reset_cg.argtypes = [vp]
        L.imdgpu_cg_step.argtypes = [vp, C.c_int]
        L.imdgpu_cg_relax.argtypes = [vp, C.c_double, C.c_int, _ip, _dp]
        L.imdgpu_get_pairs.argtypes = [vp, C.c_long, _ip, _ip, _ip, _dp,
                                       C.POINTER(C.c_long)]
        L.imdgpu_get_timing.argtypes = [vp, C.POINTER(Timing)]
        L.imdgpu_set_profiling.argtypes = [vp, C.c_int]
        L.imdgpu_device_count.argtypes = [_ip]
        L.imdgpu_put_state.argtypes = [vp, _dp, _dp]
        L.imdgpu_nve_step_host.argtypes = [vp, _dp, _dp, C.c_double, _dp, _dp,
                                           C.POINTER(Scalars)]
        L.imdgpu_set_l2_flush.argtypes = [vp, C.c_long]
        L.imdgpu_probe_fp64_peak.argtypes = [_dp]
        L.imdgpu_set_device.argtypes = [C.c_int]
        L.imdgpu_batch_set_cells.argtypes = [vp, C.c_int, _ip, _dp, _ip, _ip, _dp, _dp]
        L.imdgpu_batch_set_margin.argtypes = [vp, C.c_double]
        L.imdgpu_batch_relax.argtypes = [vp, C.c_double, C.c_int, C.c_int, _ip]
        L.imdgpu_batch_results.argtypes = [vp, _dp, _dp, _ip, _ip, _ip]
        L.imdgpu_batch_begin.argtypes = [vp, C.c_double, C.c_int]
        L.imdgpu_batch_advance.argtypes = [vp, C.c_int, _ip, _ip]
        L.imdgpu_batch_rebuilds.argtypes = [vp, C.POINTER(C.c_long)]
        L.imdgpu_batch_progress.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_long)]
        L.imdgpu_batch_set_compaction.argtypes = [vp, C.c_int]
        L.imdgpu_autotune.argtypes = [vp, _ip, _ip]
        L.imdgpu_calc_stress.argtypes = [vp, _dp, _dp]
        L.imdgpu_move_atoms_mik.argtypes = [vp, C.c_double]
        L.imdgpu_move_atoms_nvt.argtypes = [vp, C.c_double]
        L.imdgpu_set_nvt.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_long]
        L.imdgpu_get_nvt.argtypes = [vp, _dp]
        L.imdgpu_glok_defaults.argtypes = [C.POINTER(GlokParams)]
        L.imdgpu_set_glok.argtypes = [vp, C.POINTER(GlokParams), C.c_double]
        L.imdgpu_move_atoms_glok.argtypes = [vp, C.c_int]
        L.imdgpu_get_glok.argtypes = [vp, C.POINTER(GlokState)]
        L.imdgpu_npt_defaults.argtypes = [C.POINTER(NptParams)]
        L.imdgpu_set_npt.argtypes = [vp, C.POINTER(NptParams)]
        L.imdgpu_move_atoms_npt_iso.argtypes = [vp, C.c_int, C.c_double]
        L.imdgpu_get_npt.argtypes = [vp, C.POINTER(NptState)]
        L.imdgpu_npt_axial_defaults.argtypes = [C.POINTER(NptAxialParams)]
        L.imdgpu_set_npt_axial.argtypes = [vp, C.POINTER(NptAxialParams)]
        L.imdgpu_move_atoms_npt_axial.argtypes = [vp, C.c_int, C.c_double]
        L.imdgpu_get_npt_axial.argtypes = [vp, C.POINTER(NptAxialState)]
        L.imdgpu_set_blocks.argtypes = [vp, C.c_int, C.c_int]
        L.imdgpu_batch_set_autotune.argtypes = [vp, C.c_int]
        L.imdgpu_batch_set_engine.argtypes = [vp, C.c_int]
        L.imdgpu_batch_set_partial_rebuild.argtypes = [vp, C.c_int]
        L.imdgpu_batch_set_list_headroom.argtypes = [vp, C.c_double]
        L.imdgpu_batch_replays.argtypes = [vp, C.POINTER(C.c_long)]
        L.imdgpu_batch_inject_replays.argtypes = [vp, C.c_int, C.c_int]
        L.imdgpu_check_sites.argtypes = [vp, _ip, _ip]
        L.imdgpu_ml_set_tensor_cores.argtypes = [vp, C.c_int]
        L.imdgpu_batch_positions.argtypes = [vp, _dp]
        fp = C.POINTER(C.c_float)
        L.imdgpu_ml_nparam.argtypes = []
        L.imdgpu_ml_set_weights.argtypes = [vp, fp, C.c_int]
        L.imdgpu_ml_get_weights.argtypes = [vp, fp, C.c_int]
        L.imdgpu_ml_predict.argtypes = [vp, _dp]
        L.imdgpu_ml_train_step.argtypes = [vp, _dp, C.c_double, _dp, fp]
        L.imdgpu_batch_ml_start.argtypes = [vp, _ip, _dp, _dp]
        L.imdgpu_ml_get_adam.argtypes = [vp, fp, fp, _ip]
        L.imdgpu_ml_set_adam.argtypes = [vp, fp, fp, C.c_int]
        L.imdgpu_ml_set_loss_weights.argtypes = [vp, _dp]
        _lib = L
    return _lib


def _check(rc: int, what: str) -> int:
    if rc < 0:
        raise IMDGPUError("%s failed (%d): %s" % (what, rc, lib().imdgpu_last_error().decode()))
    return rc


def _p(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


class GpuSystem:
    """One simulation cell resident on the GPU.

    Tables are IMD potential files (formats 1/2) or in-memory pot_table_t
    arrays; the box, periodicity and list margin as IMD's parameters
    box_x/y/z, pbc_dirs and nbl_margin."""

    def __init__(self, ntypes: int = 1, interaction: int = EAM2, precision: int = FP64,
                 interpolation: int = QUADRATIC):
        h = C.c_void_p()
        _check(lib().imdgpu_create(C.byref(h), ntypes, interaction, precision), "imdgpu_create")
        self.h = h
        _check(lib().imdgpu_set_interpolation(h, interpolation), "set_interpolation")
        self.ntypes = ntypes
        self.interaction = interaction
        self.n = 0
        self.last_rc = 0

    # --- set-up ---------------------------------------------------------------
    def read_tables(self, files, default_format: int = 2) -> None:
        """files = (pair,) for PAIR or (pair, rho, embed) for EAM2."""
        kinds = [(TAB_PAIR, 1)] if self.interaction == PAIR else \
            [(TAB_PAIR, 1), (TAB_RHO, 1), (TAB_EMBED, 0)]
        for (which, radial), f in zip(kinds, files):
            _check(lib().imdgpu_read_table(self.h, which, f.encode(), radial, default_format),
                   "imdgpu_read_table(%s)" % f)

    def set_table(self, which, begin, end, step, length, table, maxsteps) -> None:
        ncols = len(begin)
        b, e, s = _f64(begin), _f64(end), _f64(step)
        inv = 1.0 / s
        ln = np.ascontiguousarray(length, np.int32)
        t = _f64(table)
        _check(lib().imdgpu_set_table(self.h, which, ncols, maxsteps, _p(b), _p(e), _p(s),
                                      _p(inv), _p(ln, C.c_int), _p(t)), "imdgpu_set_table")

    def set_box(self, box, pbc=(1, 1, 1), nbl_margin: float = 0.4, list_r2: float = 0.0) -> None:
        b = _f64(box, (9,))
        p = np.ascontiguousarray(pbc, np.int32)
        _check(lib().imdgpu_set_box(self.h, _p(b), _p(p, C.c_int), nbl_margin, list_r2),
               "imdgpu_set_box")

    def set_restrictions(self, restr) -> None:
        r = _f64(restr, (-1,))
        _check(lib().imdgpu_set_restrictions(self.h, _p(r)), "imdgpu_set_restrictions")

    def set_atoms(self, number, types, mass, x, p=None) -> None:
        n = len(x)
        num = np.ascontiguousarray(number, np.int32)
        ty = np.ascontiguousarray(types, np.int32)
        m = _f64(mass)
        xx = _f64(x, (n * 3,))
        pp = None if p is None else _f64(p, (n * 3,))
        _check(lib().imdgpu_set_atoms(self.h, n, _p(num, C.c_int), _p(ty, C.c_int), _p(m),
                                      _p(xx), _p(pp)), "imdgpu_set_atoms")
        self.n = n

    def put_state(self, x, p=None) -> None:
        """Positions / momenta in caller order; x, p should be C-contiguous
        float64 (pinned host memory gives direct DMA)."""
        _check(lib().imdgpu_put_state(self.h, _p(x), _p(p)), "put_state")

    def nve_step_host(self, x, p, timestep: float, x_out=None, p_out=None) -> Scalars:
        """One NVE step with the state on the host (imdgpu_nve_step_host):
        x, p up, calc_forces, move_atoms_nve with the list check, the new x, p
        into x_out / p_out (may be x, p) and the step's scalars; one
        synchronisation.  C-contiguous float64 arrays, pinned for direct DMA."""
        sc = Scalars()
        _check(lib().imdgpu_nve_step_host(self.h, _p(x), _p(p), float(timestep), _p(x_out),
                                          _p(p_out), C.byref(sc)), "nve_step_host")
        return sc

    def get_state(self, x=None, p=None, f=None, epot=None) -> None:
        """Fill the given preallocated (n,3)/(n,) float64 arrays."""
        _check(lib().imdgpu_get_atoms(self.h, _p(x), _p(p), _p(f), _p(epot), None, None),
               "get_atoms")

    def set_l2_flush(self, nbytes: int) -> None:
        _check(lib().imdgpu_set_l2_flush(self.h, nbytes), "set_l2_flush")

    def set_profiling(self, on: bool) -> None:
        _check(lib().imdgpu_set_profiling(self.h, int(on)), "set_profiling")

    def set_graphs(self, on: bool) -> None:
        """Replay NVE chunks from a captured CUDA graph (default on)."""
        _check(lib().imdgpu_set_graphs(self.h, int(on)), "set_graphs")

    def set_pair_cache(self, on: bool) -> None:
        """FP64 one-species EAM2 on one table grid: the density pass caches
        every pair's table terms for the force pass (default on)."""
        _check(lib().imdgpu_set_pair_cache(self.h, int(on)), "set_pair_cache")

    def set_table_staging(self, on: bool) -> None:
        """Mixed force pass: fused table rows staged in shared memory
        (default on) or read from global memory."""
        _check(lib().imdgpu_set_table_staging(self.h, int(on)), "set_table_staging")

    def set_exact(self, on: bool) -> None:
        """IMD's unfused table arithmetic (bitwise table values) on/off."""
        _check(lib().imdgpu_set_exact(self.h, int(on)), "set_exact")

    def format_atoms(self, flags: int, order=None) -> bytes:
        """IMD's checkpoint atom lines formatted on the device
        (imdgpu_format_atoms); order: caller indices of the lines."""
        n = 0
        op = None
        if order is not None:
            o = np.ascontiguousarray(order, np.int32)
            n = len(o)
            op = _p(o, C.c_int)
        ln = C.c_long(0)
        _check(lib().imdgpu_format_atoms(self.h, flags, op, n, None, 0, C.byref(ln)),
               "format_atoms")
        buf = C.create_string_buffer(ln.value + 1)
        _check(lib().imdgpu_format_atoms(self.h, flags, op, n, buf, ln.value, C.byref(ln)),
               "format_atoms")
        return buf.raw[:ln.value]

    def set_deterministic(self, on: bool) -> None:
        """FP64 passes on the full list without atomics: bitwise repeatable."""
        _check(lib().imdgpu_set_deterministic(self.h, int(on)), "set_deterministic")

    def set_precision(self, precision: int) -> None:
        _check(lib().imdgpu_set_precision(self.h, precision), "imdgpu_set_precision")

    # --- the hot path -----------------------------------------------------------
    def calc_forces(self, steps: int = 0) -> int:
        self.last_rc = _check(lib().imdgpu_calc_forces(self.h, steps), "calc_forces")
        return self.last_rc

    def calc_stress(self):
        """Forces plus IMD's per-atom stress (STRESS_TENS): returns
        (presstens (n, 6: xx yy zz yz zx xy), total (6,))."""
        st = np.empty((self.n, 6))
        tot = np.empty(6)
        rc = lib().imdgpu_calc_stress(self.h, _p(st), _p(tot))
        if rc < 0:
            _check(rc, "calc_stress")
        return st, tot

    def make_nblist(self) -> None:
        _check(lib().imdgpu_make_nblist(self.h), "make_nblist")

    def check_nblist(self) -> bool:
        _check(lib().imdgpu_check_nblist(self.h), "check_nblist")
        return bool(self.scalars().have_valid_nbl)

    def deallocate_nblist(self) -> None:
        _check(lib().imdgpu_deallocate_nblist(self.h), "deallocate_nblist")

    def estimate_nblist_size(self) -> int:
        n = C.c_long(0)
        _check(lib().imdgpu_estimate_nblist_size(self.h, C.byref(n)), "estimate_nblist_size")
        return n.value

    def move_atoms_nve(self, timestep: float) -> None:
        _check(lib().imdgpu_move_atoms_nve(self.h, timestep), "move_atoms_nve")

    def move_atoms_mik(self, timestep: float) -> None:
        _check(lib().imdgpu_move_atoms_mik(self.h, timestep), "move_atoms_mik")

    def set_nvt(self, temperature: float, isq_tau_eta: float, eta: float = 0.0,
                nactive: int = 0) -> None:
        _check(lib().imdgpu_set_nvt(self.h, temperature, isq_tau_eta, eta, nactive), "set_nvt")

    def move_atoms_nvt(self, timestep: float) -> float:
        """One Nose-Hoover step of the atoms; returns eta after it."""
        _check(lib().imdgpu_move_atoms_nvt(self.h, timestep), "move_atoms_nvt")
        e = C.c_double(0.0)
        _check(lib().imdgpu_get_nvt(self.h, C.byref(e)), "get_nvt")
        return e.value

    def set_glok(self, timestep: float, **params) -> None:
        """Start a glok (FIRE) phase.  params: mix, adapt (the MIX and
        ADAPTGLOK build options), glok_* and min_nPxF as IMD names them,
        steps_min, nactive; IMD's defaults for the rest."""
        prm = GlokParams()
        _check(lib().imdgpu_glok_defaults(C.byref(prm)), "glok_defaults")
        for k, v in params.items():
            if not hasattr(prm, k):
                raise TypeError("unknown glok parameter %r" % k)
            setattr(prm, k, v)
        _check(lib().imdgpu_set_glok(self.h, C.byref(prm), timestep), "set_glok")

    def move_atoms_glok(self, steps: int) -> GlokState:
        """update_glok for main_loop step `steps`, then move_atoms_nve of
        the glok ensemble; returns the glok state after it."""
        _check(lib().imdgpu_move_atoms_glok(self.h, steps), "move_atoms_glok")
        return self.glok_state()

    def relax_glok(self, timestep: float, maxsteps: int, fnorm_threshold: float = 0.0,
                   ekin_threshold: float = 0.0, delta_epot_threshold: float = 0.0,
                   steps_min: int = 0, **params):
        """main_loop of `ensemble glok` with IMD's relaxation test: per step
        calc_forces, update_glok + move_atoms_nve, check_relaxed
        (src/imd_main_3d.c:1741-1820), check_nblist; the loop ends after the
        first step that check_relaxed calls relaxed (sqrt(fnorm/nactive),
        2 E_kin/nactive or the change of E_pot per atom below its
        threshold).  Returns (steps run, relaxed)."""
        self.set_glok(timestep, steps_min=steps_min, **params)
        nact = float(params.get("nactive", 0) or 3 * self.n)
        old_epot = 0.0
        for steps in range(steps_min, steps_min + maxsteps):
            self.calc_forces(steps)
            self.move_atoms_glok(steps)
            sc = self.scalars()
            fnorm2 = np.sqrt(sc.fnorm / nact)
            ekin = 2 * sc.tot_kin_energy / nact
            epot = sc.tot_pot_energy / self.n
            delta_epot = abs(old_epot - epot)
            relaxed = (ekin < ekin_threshold or fnorm2 < fnorm_threshold
                       or delta_epot < delta_epot_threshold)
            old_epot = epot
            self.check_nblist()
            if relaxed:
                return steps - steps_min + 1, True
        return maxsteps, False

    def set_npt(self, **params) -> None:
        """Start an npt_iso phase.  params: temperature, isq_tau_eta, eta,
        isq_tau_xi, xi, pressure_ext (IMD's pressure_start), pressure_end,
        use_curr_pressure, steps_min, steps_max, nactive,
        cell_size_tolerance; IMD's defaults for the rest."""
        prm = NptParams()
        _check(lib().imdgpu_npt_defaults(C.byref(prm)), "npt_defaults")
        for k, v in params.items():
            if not hasattr(prm, k):
                raise TypeError("unknown npt parameter %r" % k)
            setattr(prm, k, v)
        _check(lib().imdgpu_set_npt(self.h, C.byref(prm)), "set_npt")

    def move_atoms_npt_iso(self, steps: int, timestep: float) -> NptState:
        """move_atoms_npt_iso for main_loop step `steps`; returns the NPT
        state after it (xi, eta, pressure, pressure_ext, volume, box)."""
        _check(lib().imdgpu_move_atoms_npt_iso(self.h, steps, timestep), "move_atoms_npt_iso")
        return self.npt_state()

    def npt_state(self) -> NptState:
        st = NptState()
        _check(lib().imdgpu_get_npt(self.h, C.byref(st)), "get_npt")
        return st

    def set_npt_axial(self, **params) -> None:
        """Start an npt_axial phase.  params: temperature, isq_tau_eta, eta,
        isq_tau_xi, xi (3), pressure_ext (3, IMD's pressure_start),
        pressure_end (3), relax_dirs (3), use_curr_pressure, steps_min,
        steps_max, nactive, cell_size_tolerance; IMD's defaults for the
        rest."""
        prm = NptAxialParams()
        _check(lib().imdgpu_npt_axial_defaults(C.byref(prm)), "npt_axial_defaults")
        for k, v in params.items():
            if not hasattr(prm, k):
                raise TypeError("unknown npt_axial parameter %r" % k)
            cur = getattr(prm, k)
            if isinstance(cur, C.Array):
                for a in range(3):
                    cur[a] = v[a]
            else:
                setattr(prm, k, v)
        _check(lib().imdgpu_set_npt_axial(self.h, C.byref(prm)), "set_npt_axial")

    def move_atoms_npt_axial(self, steps: int, timestep: float) -> NptAxialState:
        """move_atoms_npt_axial for main_loop step `steps`; returns the state
        after it (xi, eta, stress, pressure_ext, vir_axial, volume, box)."""
        _check(lib().imdgpu_move_atoms_npt_axial(self.h, steps, timestep),
               "move_atoms_npt_axial")
        return self.npt_axial_state()

    def npt_axial_state(self) -> NptAxialState:
        st = NptAxialState()
        _check(lib().imdgpu_get_npt_axial(self.h, C.byref(st)), "get_npt_axial")
        return st

    def glok_state(self) -> GlokState:
        st = GlokState()
        _check(lib().imdgpu_get_glok(self.h, C.byref(st)), "get_glok")
        return st

    def nve_run(self, nsteps: int, timestep: float, record: bool = True):
        ep = np.empty(nsteps) if record else None
        ek = np.empty(nsteps) if record else None
        self.last_rc = _check(lib().imdgpu_nve_run(self.h, nsteps, timestep, _p(ep), _p(ek)),
                              "nve_run")
        return ep, ek

    # --- CG -------------------------------------------------------------------
    def set_cg_params(self, linmin_maxsteps=100, linmin_tol=0.0002, linmin_dmax=0.01,
                      linmin_dmin=0.001, cg_glimit=100.0, cg_zeps=1e-10, cg_fr=0,
                      cg_reset_int=0) -> None:
        _check(lib().imdgpu_set_cg_params(self.h, linmin_maxsteps, linmin_tol, linmin_dmax,
                                          linmin_dmin, cg_glimit, cg_zeps, cg_fr,
                                          cg_reset_int), "set_cg_params")

    def reset_cg(self) -> None:
        _check(lib().imdgpu_reset_cg(self.h), "reset_cg")

    def cg_step(self, steps: int) -> None:
        _check(lib().imdgpu_cg_step(self.h, steps), "cg_step")

    def cg_relax(self, fmax: float = 1e-4, maxsteps: int = 100000):
        st = C.c_int(0)
        fm = C.c_double(0.0)
        _check(lib().imdgpu_cg_relax(self.h, fmax, maxsteps, C.byref(st), C.byref(fm)),
               "cg_relax")
        return st.value, fm.value

    # --- results ----------------------------------------------------------------
    def scalars(self) -> Scalars:
        s = Scalars()
        _check(lib().imdgpu_get_scalars(self.h, C.byref(s)), "get_scalars")
        return s

    def get_atoms(self):
        n = self.n
        x = np.empty((n, 3))
        p = np.empty((n, 3))
        f = np.empty((n, 3))
        e = np.empty(n)
        rho = np.empty(n)
        df = np.empty(n)
        _check(lib().imdgpu_get_atoms(self.h, _p(x), _p(p), _p(f), _p(e), _p(rho), _p(df)),
               "get_atoms")
        return {"x": x, "p": p, "f": f, "epot": e, "rho": rho, "df": df}

    def pairs(self):
        cnt = C.c_long(0)
        _check(lib().imdgpu_get_pairs(self.h, 0, None, None, None, None, C.byref(cnt)),
               "get_pairs")
        m = cnt.value
        ni = np.empty(m, np.int32)
        nj = np.empty(m, np.int32)
        sh = np.empty((m, 3), np.int32)
        r2 = np.empty(m)
        _check(lib().imdgpu_get_pairs(self.h, m, _p(ni, C.c_int), _p(nj, C.c_int),
                                      _p(sh, C.c_int), _p(r2), C.byref(cnt)), "get_pairs")
        return ni, nj, sh, r2

    # --- learned start ---------------------------------------------------------
    def ml_set_tensor_cores(self, on: bool) -> None:
        """Forward pass on tcgen05 instead of mma.sync
        (imdgpu_ml_set_tensor_cores)."""
        _check(lib().imdgpu_ml_set_tensor_cores(self.h, int(bool(on))), "ml_set_tensor_cores")

    def ml_set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        _check(lib().imdgpu_ml_set_weights(self.h, _p(w, C.c_float), len(w)), "ml_set_weights")

    def ml_get_weights(self):
        w = np.empty(lib().imdgpu_ml_nparam(), np.float32)
        _check(lib().imdgpu_ml_get_weights(self.h, _p(w, C.c_float), len(w)), "ml_get_weights")
        return w

    def ml_get_adam(self):
        """(m, v, step): the Adam state of the weights."""
        k = lib().imdgpu_ml_nparam()
        m = np.empty(k, np.float32)
        v = np.empty(k, np.float32)
        t = C.c_int(0)
        _check(lib().imdgpu_ml_get_adam(self.h, _p(m, C.c_float), _p(v, C.c_float),
                                        C.byref(t)), "ml_get_adam")
        return m, v, t.value

    def ml_set_adam(self, m, v, step: int) -> None:
        m = np.ascontiguousarray(m, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        _check(lib().imdgpu_ml_set_adam(self.h, _p(m, C.c_float), _p(v, C.c_float), int(step)),
               "ml_set_adam")

    def ml_predict(self):
        """Predicted displacements (n,3), caller order, at the current positions."""
        dx = np.empty((self.n, 3))
        _check(lib().imdgpu_ml_predict(self.h, _p(dx)), "ml_predict")
        return dx

    def ml_set_loss_weights(self, w=None) -> None:
        """Per-atom weights of the training loss (caller order); None: all 1."""
        if w is None:
            _check(lib().imdgpu_ml_set_loss_weights(self.h, None), "ml_set_loss_weights")
            return
        w = _f64(w, (self.n,))
        _check(lib().imdgpu_ml_set_loss_weights(self.h, _p(w)), "ml_set_loss_weights")

    def ml_train_step(self, target, lr: float = 0.0, want_grad: bool = False):
        """Loss (and gradient) for per-atom target displacements; with lr > 0
        one Adam step of the weights."""
        t = _f64(target, (self.n * 3,))
        loss = C.c_double(0.0)
        g = np.empty(lib().imdgpu_ml_nparam(), np.float32) if want_grad else None
        _check(lib().imdgpu_ml_train_step(self.h, _p(t), lr, C.byref(loss),
                                          _p(g, C.c_float)), "ml_train_step")
        return (loss.value, g) if want_grad else loss.value

    def autotune(self):
        """Pick the density and force passes' blocks by timing; returns both."""
        bd = C.c_int(0)
        bf = C.c_int(0)
        _check(lib().imdgpu_autotune(self.h, C.byref(bd), C.byref(bf)), "autotune")
        return bd.value, bf.value

    def tile(self) -> int:
        """Lanes per atom the autotuner chose (imdgpu_get_tile)."""
        t = C.c_int(0)
        _check(lib().imdgpu_get_tile(self.h, C.byref(t)), "get_tile")
        return t.value

    def set_blocks(self, density: int, force: int) -> None:
        _check(lib().imdgpu_set_blocks(self.h, int(density), int(force)), "set_blocks")

    def timing(self) -> Timing:
        t = Timing()
        _check(lib().imdgpu_get_timing(self.h, C.byref(t)), "get_timing")
        return t

    def check_sites(self):
        """(checked, sites): whether the loaded library is the bounds-checked
        build, and the mask of the checks that failed (imdgpu_check_sites)."""
        c, m = C.c_int(0), C.c_int(0)
        _check(lib().imdgpu_check_sites(self.h, C.byref(c), C.byref(m)), "check_sites")
        return bool(c.value), m.value

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().imdgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuBatch(GpuSystem):
    """Many independent periodic cells relaxed together by IMD's CG, one
    line-search state per cell on the device (imdgpu_batch_* in
    include/imdgpu.h)."""

    def set_cells(self, cells, nbl_margin: float = 0.4) -> None:
        """cells: sequence of workloads.System (box, x, types, mass, number)."""
        natoms = np.array([c.n for c in cells], np.int32)
        boxes = np.ascontiguousarray(np.stack([np.asarray(c.box, np.float64) for c in cells]))
        x = np.ascontiguousarray(np.concatenate([c.x for c in cells]), np.float64)
        ty = np.ascontiguousarray(np.concatenate([c.types for c in cells]), np.int32)
        m = np.ascontiguousarray(np.concatenate([c.mass for c in cells]), np.float64)
        num = np.ascontiguousarray(np.concatenate([c.number for c in cells]), np.int32)
        _check(lib().imdgpu_batch_set_margin(self.h, nbl_margin), "batch_set_margin")
        _check(lib().imdgpu_batch_set_cells(self.h, len(cells), _p(natoms, C.c_int), _p(boxes),
                                            _p(num, C.c_int), _p(ty, C.c_int), _p(m), _p(x)),
               "batch_set_cells")
        self.n = int(natoms.sum())
        self.ncells = len(cells)
        self.natoms = natoms

    def relax(self, fmax: float = 1e-4, maxsteps: int = 100000, max_rounds: int = 1000000) -> int:
        r = C.c_int(0)
        _check(lib().imdgpu_batch_relax(self.h, fmax, maxsteps, max_rounds, C.byref(r)),
               "batch_relax")
        return r.value

    def begin(self, fmax: float = 1e-4, maxsteps: int = 100000) -> None:
        _check(lib().imdgpu_batch_begin(self.h, fmax, maxsteps), "batch_begin")

    def advance(self, max_rounds: int):
        nd = C.c_int(0)
        r = C.c_int(0)
        _check(lib().imdgpu_batch_advance(self.h, max_rounds, C.byref(nd), C.byref(r)),
               "batch_advance")
        return nd.value, r.value

    def ml_start(self):
        """Learned start (weights set with ml_set_weights): every cell keeps
        its predicted positions where they lower its energy.  Returns
        (used, e_start, e_pred) per cell."""
        k = self.ncells
        used = np.empty(k, np.int32)
        e0 = np.empty(k)
        e1 = np.empty(k)
        _check(lib().imdgpu_batch_ml_start(self.h, _p(used, C.c_int), _p(e0), _p(e1)),
               "batch_ml_start")
        return used, e0, e1

    def rebuilds(self) -> int:
        n = C.c_long(0)
        _check(lib().imdgpu_batch_rebuilds(self.h, C.byref(n)), "batch_rebuilds")
        return n.value

    def progress(self):
        """(cells finished, atoms of the unfinished cells)."""
        nd = C.c_int(0)
        a = C.c_long(0)
        _check(lib().imdgpu_batch_progress(self.h, C.byref(nd), C.byref(a)), "batch_progress")
        return nd.value, a.value

    def results(self):
        k = self.ncells
        e = np.empty(k)
        fm = np.empty(k)
        st = np.empty(k, np.int32)
        nfc = np.empty(k, np.int32)
        status = np.empty(k, np.int32)
        _check(lib().imdgpu_batch_results(self.h, _p(e), _p(fm), _p(st, C.c_int),
                                          _p(nfc, C.c_int), _p(status, C.c_int)), "batch_results")
        return {"epot": e, "fmax": fm, "steps": st, "nfc": nfc, "status": status}

    def positions(self):
        """Current positions, one (n_c, 3) array per cell."""
        x = np.empty((self.n, 3))
        _check(lib().imdgpu_batch_positions(self.h, _p(x)), "batch_positions")
        return np.split(x, np.cumsum(self.natoms)[:-1])

    def set_engine(self, on: bool) -> None:
        """A round's CG work in one persistent kernel (default on) or in four
        kernels (imdgpu_batch_set_engine)."""
        _check(lib().imdgpu_batch_set_engine(self.h, int(bool(on))), "batch_set_engine")

    def set_list_headroom(self, factor: float) -> None:
        """List capacity over the largest count at a build (default 1.3)."""
        _check(lib().imdgpu_batch_set_list_headroom(self.h, float(factor)),
               "batch_set_list_headroom")

    def replays(self) -> int:
        """Chunks of rounds replayed after an overflow since begin()."""
        n = C.c_long(0)
        _check(lib().imdgpu_batch_replays(self.h, C.byref(n)), "batch_replays")
        return n.value

    def inject_replays(self, every: int, count: int) -> None:
        """Test hook: after every `every` completed chunks the next chunk is
        replayed from its snapshot as after an overflow, `count` times in all
        (imdgpu_batch_inject_replays; call after begin())."""
        _check(lib().imdgpu_batch_inject_replays(self.h, int(every), int(count)),
               "batch_inject_replays")

    def set_partial_rebuild(self, on: bool) -> None:
        """Rebuild the lists of the cells that moved only, each cell with a
        fixed ghost range (imdgpu_batch_set_partial_rebuild)."""
        _check(lib().imdgpu_batch_set_partial_rebuild(self.h, int(bool(on))),
               "batch_set_partial_rebuild")

    def set_autotune(self, on: bool) -> None:
        """Tune the block shape at every imdgpu_batch_begin (default on)."""
        _check(lib().imdgpu_batch_set_autotune(self.h, int(bool(on))), "batch_set_autotune")

    def set_compaction(self, pct: int) -> None:
        """Drop finished cells from the device once the unfinished ones hold
        at most pct % of its atoms (0: never)."""
        _check(lib().imdgpu_batch_set_compaction(self.h, int(pct)), "batch_set_compaction")


FMT_HPO, FMT_VELOCITY, FMT_EAM_RHO = 1, 2, 4


def format_fixed(x, prec: int, width: int = 0) -> bytes:
    """Each value as printf("%*.*f\\n", width, prec, v), formatted on the
    device (imdgpu_format_fixed)."""
    a = np.ascontiguousarray(x, np.float64)
    ln = C.c_long(0)
    _check(lib().imdgpu_format_fixed(_p(a), len(a), prec, width, None, 0, C.byref(ln)),
           "format_fixed")
    buf = C.create_string_buffer(ln.value + 1)
    _check(lib().imdgpu_format_fixed(_p(a), len(a), prec, width, buf, ln.value, C.byref(ln)),
           "format_fixed")
    return buf.raw[:ln.value]


def set_device(device: int) -> None:
    _check(lib().imdgpu_set_device(device), "set_device")


def probe_fp64_peak() -> float:
    """Measured FP64 FMA throughput of the current device in TFLOP/s."""
    v = C.c_double(0.0)
    _check(lib().imdgpu_probe_fp64_peak(C.byref(v)), "probe_fp64_peak")
    return v.value


def system_from_tables(files, box, number, types, mass, x, p=None, ntypes=1,
                       interaction=EAM2, precision=FP64, nbl_margin=0.4, pbc=(1, 1, 1)):
    """Convenience: a GpuSystem with tables, box and atoms set."""
    s = GpuSystem(ntypes, interaction, precision)
    s.read_tables(files)
    s.set_box(box, pbc, nbl_margin)
    s.set_atoms(number, types, mass, x, p)
    return s
