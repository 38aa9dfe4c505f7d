"""ctypes binding of the C oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and the CPU
baseline arm of bench.py import this module.  It is the oracle, never the
thing measured on the GPU and never called by imd_gb300.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Table(C.Structure):
    _fields_ = [("ncols", C.c_int), ("maxsteps", C.c_int), ("begin", _dp), ("end", _dp),
                ("step", _dp), ("invstep", _dp), ("len", _ip), ("table", _dp),
                ("table2", _dp), ("mode", C.c_int)]

QUADRATIC, FOURPOINT, SPLINE = 0, 1, 2


def set_interpolation(mode: int) -> None:
    """How tables read afterwards are initialised and interpolated."""
    lib().orc_set_interpolation(mode)


class Sys(C.Structure):
    _fields_ = [
        ("ntypes", C.c_int), ("interaction", C.c_int), ("box", (C.c_double * 3) * 3),
        ("pbc", C.c_int * 3), ("nbl_margin", C.c_double), ("timestep", C.c_double),
        ("restrictions", _dp), ("linmin_maxsteps", C.c_int), ("linmin_tol", C.c_double),
        ("linmin_dmax", C.c_double), ("linmin_dmin", C.c_double), ("cg_glimit", C.c_double),
        ("cg_zeps", C.c_double), ("cg_fr", C.c_int), ("cg_reset_int", C.c_int),
        ("cg_brent_full", C.c_int),
        ("pair", Table), ("rho", Table), ("embed", Table), ("cellsz", C.c_double),
        ("n", C.c_int), ("number", _ip), ("type", _ip), ("mass", _dp), ("x", _dp),
        ("p", _dp), ("f", _dp), ("epot", _dp), ("eam_rho", _dp), ("eam_df", _dp),
        ("nbl_pos", _dp), ("tbox", (C.c_double * 3) * 3), ("volume", C.c_double),
        ("height", C.c_double * 3), ("gdim", C.c_int * 3), ("cdim", C.c_int * 3),
        ("nallcells", C.c_int), ("nreal_cells", C.c_int), ("real_cells", _ip),
        ("cnbrs", _ip), ("cell_start", _ip), ("cell_cnt", _ip), ("cell_atoms", _ip),
        ("next", C.c_int), ("next_cap", C.c_int), ("ex", _dp), ("etype", _ip),
        ("esrc", _ip), ("eowner", _ip), ("eshift", _dp), ("ef", _dp), ("eepot", _dp),
        ("erho", _dp), ("edf", _dp), ("order", _ip), ("tl", _ip), ("tb", _ip),
        ("nb_cap", C.c_long), ("nb_len", C.c_long), ("have_valid_nbl", C.c_int),
        ("nbl_count", C.c_long), ("nfc", C.c_long), ("is_short", C.c_int),
        ("tot_pot_energy", C.c_double), ("virial", C.c_double),
        ("tot_kin_energy", C.c_double), ("fnorm", C.c_double), ("f_max2", C.c_double),
        ("old_x", _dp), ("cg_g", _dp), ("cg_h", _dp), ("cg_gamma", C.c_double),
        ("cg_poteng", C.c_double), ("old_cg_poteng", C.c_double),
        ("old_alphamin", C.c_double), ("nactive", C.c_long),
        ("do_stress", C.c_int), ("estress", _dp), ("stress", _dp),
        ("tot_stress", C.c_double * 6),
        ("eta", C.c_double), ("isq_tau_eta", C.c_double), ("temperature", C.c_double),
        ("vir_axial", C.c_double * 3), ("tot_pot_energy_c", C.c_double),
        ("virial_c", C.c_double)]


class Glok(C.Structure):
    """orc_glok_t: parameters and state of the glok ensemble."""
    _fields_ = [("mix_on", C.c_int), ("adapt", C.c_int), ("glok_ekin_threshold", C.c_double),
                ("glok_fmaxcrit", C.c_double), ("glok_mix", C.c_double),
                ("glok_mixdec", C.c_double), ("glok_incfac", C.c_double),
                ("glok_decfac", C.c_double), ("glok_maxtimestep", C.c_double),
                ("glok_minsteps", C.c_int), ("min_nPxF", C.c_int), ("steps_min", C.c_int),
                ("nactive", C.c_long), ("glok_start", C.c_int), ("glok_int", C.c_int),
                ("nPxF", C.c_int), ("mix", C.c_double), ("mixforcescalefac", C.c_double),
                ("PxF", C.c_double), ("pnorm", C.c_double)]


class Npt(C.Structure):
    """orc_npt_t: parameters and state of ensemble npt_iso."""
    _fields_ = [("temperature", C.c_double), ("isq_tau_eta", C.c_double), ("eta", C.c_double),
                ("isq_tau_xi", C.c_double), ("xi", C.c_double), ("xi_old", C.c_double),
                ("pressure_ext", C.c_double), ("pressure_end", C.c_double),
                ("pressure", C.c_double), ("d_pressure", C.c_double), ("Ekin_old", C.c_double),
                ("volume_init", C.c_double), ("cell_size_tolerance", C.c_double), ("min_height", C.c_double * 3),
                ("max_height", C.c_double * 3), ("use_curr_pressure", C.c_int),
                ("steps_min", C.c_int), ("steps_max", C.c_int), ("nactive", C.c_long)]


class NptAxial(C.Structure):
    """orc_npt_axial_t: parameters and state of ensemble npt_axial."""
    _d3 = C.c_double * 3
    _fields_ = [("temperature", C.c_double), ("isq_tau_eta", C.c_double), ("eta", C.c_double),
                ("isq_tau_xi", C.c_double), ("xi", _d3), ("xi_old", _d3),
                ("pressure_ext", _d3), ("pressure_end", _d3), ("d_pressure", _d3),
                ("stress", _d3), ("dyn_stress", _d3), ("Ekin_old", C.c_double),
                ("volume_init", C.c_double), ("cell_size_tolerance", C.c_double),
                ("min_height", _d3), ("max_height", _d3), ("relax_dirs", C.c_int * 3),
                ("use_curr_pressure", C.c_int), ("steps_min", C.c_int), ("steps_max", C.c_int),
                ("nactive", C.c_long)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
        L = C.CDLL(LIB)
        L.orc_read_table.argtypes = [C.POINTER(Table), C.c_char_p, C.c_int, C.c_int, C.c_int,
                                     _dp, C.c_char_p, C.c_int]
        L.orc_pair_int2_batch.argtypes = [C.POINTER(Table), C.c_int, C.c_int, C.c_int, _dp,
                                          _dp, _dp]
        L.orc_val_func2.argtypes = [C.POINTER(Table), C.c_int, C.c_int, C.c_double, _ip]
        L.orc_val_func2.restype = C.c_double
        L.orc_deriv_func2.argtypes = [C.POINTER(Table), C.c_int, C.c_int, C.c_double, _ip]
        L.orc_deriv_func2.restype = C.c_double
        for fn in ("orc_init",):
            getattr(L, fn).argtypes = [C.POINTER(Sys), C.c_int]
        for fn in ("orc_setup_geometry", "orc_rebuild", "orc_calc_forces", "orc_reset_cg"):
            getattr(L, fn).argtypes = [C.POINTER(Sys)]
        L.orc_move_atoms_nve.argtypes = [C.POINTER(Sys)]
        L.orc_check_nblist.argtypes = [C.POINTER(Sys)]
        L.orc_free.argtypes = [C.POINTER(Sys)]
        L.orc_nve_steps.argtypes = [C.POINTER(Sys), C.c_int, _dp, _dp]
        L.orc_md_steps.argtypes = [C.POINTER(Sys), C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_glok_defaults.argtypes = [C.POINTER(Glok)]
        L.orc_npt_defaults.argtypes = [C.POINTER(Npt)]
        L.orc_npt_begin.argtypes = [C.POINTER(Sys), C.POINTER(Npt)]
        L.orc_npt_steps.argtypes = [C.POINTER(Sys), C.POINTER(Npt), C.c_int, C.c_int, _dp]
        L.orc_npt_axial_defaults.argtypes = [C.POINTER(NptAxial)]
        L.orc_npt_axial_begin.argtypes = [C.POINTER(Sys), C.POINTER(NptAxial)]
        L.orc_npt_axial_steps.argtypes = [C.POINTER(Sys), C.POINTER(NptAxial), C.c_int,
                                          C.c_int, _dp]
        L.orc_glok_steps.argtypes = [C.POINTER(Sys), C.POINTER(Glok), C.c_int, C.c_int, _dp]
        L.orc_cg_step.argtypes = [C.POINTER(Sys), C.c_int]
        L.orc_cg_relax.argtypes = [C.POINTER(Sys), C.c_double, C.c_int, _dp]
        L.orc_max_atom_force.argtypes = [C.POINTER(Sys)]
        L.orc_max_atom_force.restype = C.c_double
        L.orc_pairs.argtypes = [C.POINTER(Sys), C.c_long, _ip, _ip, _ip, _dp]
        L.orc_pairs.restype = C.c_long
        L.orc_set_interpolation.argtypes = [C.c_int]
        _lib = L
    return _lib


def _ptr(a: np.ndarray, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


class OracleTable:
    """A potential table read by the oracle's restatement of read_pot_table."""

    def __init__(self, path: str, ncols: int, radial: bool, default_format: int = 2):
        self.t = Table()
        self.cellsz = C.c_double(0.0)
        err = C.create_string_buffer(512)
        rc = lib().orc_read_table(C.byref(self.t), path.encode(), ncols, int(radial),
                                  default_format, C.byref(self.cellsz), err, 512)
        if rc:
            raise IOError(err.value.decode())

    def pair_int2(self, col: int, inc: int, r2: np.ndarray):
        r2 = np.ascontiguousarray(r2, np.float64)
        pot = np.empty_like(r2)
        grad = np.empty_like(r2)
        lib().orc_pair_int2_batch(C.byref(self.t), col, inc, len(r2), _ptr(r2), _ptr(pot),
                                  _ptr(grad))
        return pot, grad

    def val(self, col: int, inc: int, r2: float) -> float:
        s = C.c_int(0)
        return lib().orc_val_func2(C.byref(self.t), col, inc, r2, C.byref(s))

    def deriv(self, col: int, inc: int, r2: float) -> float:
        s = C.c_int(0)
        return lib().orc_deriv_func2(C.byref(self.t), col, inc, r2, C.byref(s))


class OracleSystem:
    """One simulation cell held by the oracle (atom-major arrays)."""

    def __init__(self, box, x, types, mass, number, ntypes, tables, eam: bool,
                 nbl_margin: float, timestep: float = 0.0, p=None, pbc=(1, 1, 1)):
        L = lib()
        self.s = s = Sys()
        n = len(x)
        s.ntypes = ntypes
        s.interaction = 1 if eam else 0
        for a in range(3):
            for c in range(3):
                s.box[a][c] = float(box[a][c])
            s.pbc[a] = int(pbc[a])
        s.nbl_margin = nbl_margin
        s.timestep = timestep
        cellsz = C.c_double(0.0)
        err = C.create_string_buffer(512)
        if eam:
            pt, rt, et = tables
            self._read(s.pair, pt, ntypes * ntypes, 1, cellsz, err)
            self._read(s.rho, rt, ntypes * ntypes, 1, cellsz, err)
            self._read(s.embed, et, ntypes, 0, cellsz, err)
        else:
            self._read(s.pair, tables[0], ntypes * ntypes, 1, cellsz, err)
        if L.orc_init(C.byref(s), n):
            raise MemoryError("oracle init")
        s.cellsz = cellsz.value
        self.n = n
        self._copy_in(x, types, mass, number, p)
        rc = L.orc_setup_geometry(C.byref(s))
        if rc:
            raise ValueError("oracle geometry set-up failed (%d)" % rc)

    @staticmethod
    def _read(t, path, ncols, radial, cellsz, err):
        rc = lib().orc_read_table(C.byref(t), path.encode(), ncols, radial, 2,
                                  C.byref(cellsz), err, 512)
        if rc:
            raise IOError(err.value.decode())

    def _arr(self, name, shape, dtype=np.float64):
        ptr = getattr(self.s, name)
        return np.ctypeslib.as_array(ptr, shape=shape) if dtype == np.float64 else \
            np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_int)), shape=shape)

    def _copy_in(self, x, types, mass, number, p):
        n = self.n
        self._arr("x", (n, 3))[:] = x
        self._arr("type", (n,), np.int32)[:] = types
        self._arr("mass", (n,))[:] = mass
        self._arr("number", (n,), np.int32)[:] = number
        if p is not None:
            self._arr("p", (n, 3))[:] = p

    # views
    @property
    def x(self):
        return self._arr("x", (self.n, 3))

    @property
    def p(self):
        return self._arr("p", (self.n, 3))

    @property
    def f(self):
        return self._arr("f", (self.n, 3))

    @property
    def epot(self):
        return self._arr("epot", (self.n,))

    @property
    def rho(self):
        return self._arr("eam_rho", (self.n,))

    @property
    def df(self):
        return self._arr("eam_df", (self.n,))

    @property
    def stress(self):
        """Per-atom PRESSTENS (n, 6: xx yy zz yz zx xy) of the last calc_forces
        with do_stress set."""
        return self._arr("stress", (self.n, 6))

    @property
    def tot_stress(self):
        return np.array(self.s.tot_stress[:])

    def set_stress(self, on: bool = True) -> None:
        """do_press_calc: the next calc_forces also accumulates PRESSTENS."""
        self.s.do_stress = 1 if on else 0

    @property
    def epot_total(self):
        return self.s.tot_pot_energy

    @property
    def virial(self):
        return self.s.virial

    @property
    def epot_total_exact(self):
        """tot_pot_energy by compensated summation (IMD's running sum loses
        about terms x eps relative at large N)."""
        return self.s.tot_pot_energy_c

    @property
    def virial_exact(self):
        return self.s.virial_c

    @property
    def ekin(self):
        return self.s.tot_kin_energy

    def calc_forces(self):
        lib().orc_calc_forces(C.byref(self.s))

    def invalidate(self):
        self.s.have_valid_nbl = 0

    def nve(self, nsteps: int):
        ep = np.empty(nsteps)
        ek = np.empty(nsteps)
        lib().orc_nve_steps(C.byref(self.s), nsteps, _ptr(ep), _ptr(ek))
        return ep, ek

    def md(self, nsteps: int, ensemble: str = "nve"):
        """main_loop steps with move_atoms_nve / _nvt / _mik: per step
        tot_pot_energy, tot_kin_energy and eta (nvt) or fnorm (nve, mik)."""
        code = {"nve": 0, "nvt": 1, "mik": 2}[ensemble]
        ep = np.empty(nsteps)
        ek = np.empty(nsteps)
        ex = np.empty(nsteps)
        lib().orc_md_steps(C.byref(self.s), nsteps, code, _ptr(ep), _ptr(ek), _ptr(ex))
        return ep, ek, ex

    def glok(self, nsteps: int, step0: int = 0, state: Glok = None, **params):
        """main_loop steps of the glok ensemble (update_glok, move_atoms_nve)
        from step `step0`.  params: mix_on, adapt and the glok_* values
        (IMD's defaults otherwise).  Returns (per-step array of tot_pot_energy,
        tot_kin_energy, fnorm, f_max2, timestep, mix, PxF, glok_start; the
        state, to continue with)."""
        L = lib()
        if state is None:
            state = Glok()
            L.orc_glok_defaults(C.byref(state))
            for k, v in params.items():
                setattr(state, k, v)
        out = np.empty((nsteps, 8))
        rc = L.orc_glok_steps(C.byref(self.s), C.byref(state), step0, nsteps, _ptr(out))
        if rc < 0:
            raise RuntimeError("oracle glok steps failed (%d)" % rc)
        return out, state

    def npt(self, nsteps: int, step0: int = 0, state: Npt = None, **params):
        """main_loop steps of ensemble npt_iso from step `step0`.  params:
        the orc_npt_t fields (IMD's names); a new state re-initialises the
        cell grid with the NPT tolerance as IMD does for this ensemble.
        Returns (per-step array of tot_pot_energy, tot_kin_energy, xi, eta,
        pressure, volume, box_x.x, pressure_ext; the state)."""
        L = lib()
        if state is None:
            state = Npt()
            L.orc_npt_defaults(C.byref(state))
            for k, v in params.items():
                setattr(state, k, v)
            if L.orc_npt_begin(C.byref(self.s), C.byref(state)):
                raise ValueError("oracle npt grid set-up failed")
        out = np.empty((nsteps, 8))
        rc = L.orc_npt_steps(C.byref(self.s), C.byref(state), step0, nsteps, _ptr(out))
        if rc < 0:
            raise RuntimeError("oracle npt steps failed (%d)" % rc)
        return out, state

    def npt_axial(self, nsteps: int, step0: int = 0, state: NptAxial = None, **params):
        """main_loop steps of ensemble npt_axial from step `step0`; params as
        the orc_npt_axial_t fields (3-vectors as sequences).  Returns
        (per-step array of tot_pot_energy, tot_kin_energy, xi (3), eta,
        stress (3), box diagonal (3); the state)."""
        L = lib()
        if state is None:
            state = NptAxial()
            L.orc_npt_axial_defaults(C.byref(state))
            for k, v in params.items():
                if isinstance(getattr(state, k), C.Array):
                    arr = getattr(state, k)
                    for a in range(3):
                        arr[a] = v[a]
                else:
                    setattr(state, k, v)
            if L.orc_npt_axial_begin(C.byref(self.s), C.byref(state)):
                raise ValueError("oracle npt grid set-up failed")
        out = np.empty((nsteps, 12))
        rc = L.orc_npt_axial_steps(C.byref(self.s), C.byref(state), step0, nsteps, _ptr(out))
        if rc < 0:
            raise RuntimeError("oracle npt_axial steps failed (%d)" % rc)
        return out, state

    def set_nvt(self, temperature: float, isq_tau_eta: float, eta: float = 0.0) -> None:
        self.s.temperature = temperature
        self.s.isq_tau_eta = isq_tau_eta
        self.s.eta = eta

    def cg_relax(self, fmax: float, maxsteps: int = 100000):
        fm = C.c_double(0.0)
        st = lib().orc_cg_relax(C.byref(self.s), fmax, maxsteps, C.byref(fm))
        return st, fm.value

    def raw_pairs(self):
        """Pairs of the current list in list order: NUMMER of both atoms, the
        image shift of the second (n, 3) and r^2."""
        cnt = lib().orc_pairs(C.byref(self.s), 0, None, None, None, None)
        ni = np.empty(cnt, np.int32)
        nj = np.empty(cnt, np.int32)
        sh = np.empty((cnt, 3), np.int32)
        r2 = np.empty(cnt)
        lib().orc_pairs(C.byref(self.s), cnt, _ptr(ni, C.c_int), _ptr(nj, C.c_int),
                        _ptr(sh, C.c_int), _ptr(r2))
        return ni, nj, sh, r2

    def pairs(self):
        """Canonical sorted pair keys and r2 of the current list."""
        return canonical(*self.raw_pairs())

    @property
    def nfc(self):
        return self.s.nfc

    @property
    def nbl_count(self):
        return self.s.nbl_count

    def close(self):
        if self.s is not None:
            lib().orc_free(C.byref(self.s))
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decode_keys(key):
    """Inverse of the key of canonical(): (lo, hi, shift (n, 3))."""
    key = np.asarray(key, np.int64)
    code = key % 27
    lohi = key // 27
    sh = np.stack([code // 9 - 1, (code // 3) % 3 - 1, code % 3 - 1], axis=1)
    return lohi >> 24, lohi & ((1 << 24) - 1), sh


def canonical(ni, nj, shift, r2):
    """Canonical unordered pair keys: (lo, hi, image shift of hi rel. lo),
    sorted; r2 follows the same permutation."""
    ni = np.asarray(ni, np.int64)
    nj = np.asarray(nj, np.int64)
    s = np.asarray(shift, np.int64).reshape(-1, 3)
    flip = (ni > nj) | ((ni == nj) & (
        (s[:, 0] < 0) | ((s[:, 0] == 0) & ((s[:, 1] < 0) | ((s[:, 1] == 0) & (s[:, 2] < 0))))))
    lo = np.where(flip, nj, ni)
    hi = np.where(flip, ni, nj)
    s = np.where(flip[:, None], -s, s)
    key = ((lo * (1 << 24) + hi) * 27 + (s[:, 0] + 1) * 9 + (s[:, 1] + 1) * 3 + (s[:, 2] + 1))
    order = np.argsort(key, kind="stable")
    return key[order], np.asarray(r2)[order]


def _mix64(z):
    """splitmix64 finaliser on a uint64 array (wrapping arithmetic)."""
    z = z + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def pair_digest(ni, nj, shift, r2, chunk: int = 1 << 24):
    """Order-independent digest of a pair set: (count, sum and xor over all
    pairs of a 64-bit hash of the canonical key and the bits of r^2, both
    mod 2^64).  Equal sets give equal digests whatever order the pairs come
    in, so two lists of hundreds of millions of pairs compare without a sort.
    """
    n = len(ni)
    acc_sum = np.uint64(0)
    acc_xor = np.uint64(0)
    shift = np.asarray(shift).reshape(-1, 3)
    with np.errstate(over="ignore"):
        for a in range(0, n, chunk):
            b = min(n, a + chunk)
            i = np.asarray(ni[a:b], np.int64)
            j = np.asarray(nj[a:b], np.int64)
            s = np.asarray(shift[a:b], np.int64)
            flip = (i > j) | ((i == j) & (
                (s[:, 0] < 0) | ((s[:, 0] == 0) & ((s[:, 1] < 0) | ((s[:, 1] == 0) & (s[:, 2] < 0))))))
            lo = np.where(flip, j, i)
            hi = np.where(flip, i, j)
            s = np.where(flip[:, None], -s, s)
            key = ((lo * (1 << 24) + hi) * 27 + (s[:, 0] + 1) * 9 + (s[:, 1] + 1) * 3
                   + (s[:, 2] + 1)).astype(np.uint64)
            bits = np.ascontiguousarray(r2[a:b], np.float64).view(np.uint64)
            h = _mix64(key ^ _mix64(bits))
            acc_sum = acc_sum + np.add.reduce(h, dtype=np.uint64)
            acc_xor = acc_xor ^ np.bitwise_xor.reduce(h)
    return int(n), int(acc_sum), int(acc_xor)
