"""IMD's checkpoint text formatted on the device against glibc's printf.

write_atoms_config (src/imd_io_3d.c:696-948) prints every atom with
sprintf; imdgpu_format_atoms produces the same lines on the device.  The
yardstick is the C library's own snprintf, called through ctypes on the same
doubles:

* imdgpu_format_fixed on 200,000 doubles of random magnitude (1e-17 .. 1e19)
  and on edge cases (exact ties at the last printed digit, +-0, subnormals,
  NaN, infinities), with IMD's two formats " %12.16f" (hpo) and " %f", and
  with no decimals;
* imdgpu_format_atoms on the Cu NVE workload after 20 steps (positions,
  velocities = momenta / mass, per-atom energies, rho), in caller order and
  in a shuffled order, every flag combination;
* a value of magnitude 2^63 or more is refused.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, tables

pytestmark = pytest.mark.gpu

_libc = C.CDLL(None)
_libc.snprintf.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p]


def c_fixed(v, fmt: bytes) -> bytes:
    buf = C.create_string_buffer(512)
    _libc.snprintf(buf, 512, fmt, C.c_double(float(v)))
    return buf.value


def _edge_values():
    v = [0.0, -0.0, 0.5, 1.5, 2.5, -0.5, 0.5e-16, 1.5e-16, 2.5e-16, 5e-324, -5e-324,
         float("nan"), float("inf"), -float("inf"), 9.2e18, -9.2e18, 123.45678901234567,
         0.9999999999999999, 7.5e-7, 2.5e-6, 0.0000005]
    for k in range(1, 400):
        v += [k / 2.0, k / 1024.0, k / 2 ** 20, -k / 2 ** 17, k * 0.5e-6, k * 2.0 ** -54]
    return v


@pytest.mark.parametrize("prec,width", [(16, 12), (6, 0), (0, 0)])
def test_format_fixed_equals_printf(prec, width):
    from imd_gb300 import api
    rng = np.random.default_rng(7)
    vals = rng.standard_normal(200_000) * np.exp(rng.uniform(-40, 44, 200_000))
    vals = vals[np.abs(vals) < 2.0 ** 63]
    vals = np.concatenate([vals, np.array(_edge_values())])
    got = api.format_fixed(vals, prec, width).split(b"\n")[:-1]
    fmt = ("%%%d.%df" % (width, prec)).encode()
    assert len(got) == len(vals)
    bad = [(v, g) for v, g in zip(vals, got) if g != c_fixed(v, fmt)]
    assert not bad, bad[:5]


def test_format_fixed_refuses_huge_values():
    from imd_gb300 import api
    with pytest.raises(api.IMDGPUError):
        api.format_fixed(np.array([1.0, 2.0 ** 64, 3.0]), 16, 12)


def _printf_lines(a, flags, order):
    hpo = flags & 1
    f = b" %12.16f" if hpo else b" %f"
    out = []
    for i in order:
        parts = [b"%d %d" % (a["number"][i], a["type"][i])]
        vals = [a["mass"][i], *a["x"][i]]
        if flags & 2:
            vals += [a["p"][i][c] / a["mass"][i] for c in range(3)]
        vals.append(a["epot"][i])
        if flags & 4:
            vals.append(a["rho"][i])
        parts += [c_fixed(v, f) for v in vals]
        out.append(b"".join(parts) + b"\n")
    return b"".join(out)


def test_format_atoms_equals_printf():
    from imd_gb300 import api
    g = golden("cu_nve")
    s = api.GpuSystem(1, api.EAM2, api.FP64)
    s.read_tables(tables("cu"))
    s.set_box(g["box"], (1, 1, 1), 0.4)
    s.set_atoms(g["number"], g["type"], g["mass"], g["x0"], g["p0"])
    s.nve_run(20, float(g["dt"]), record=False)
    s.calc_forces(20)
    a = s.get_atoms()
    a["number"] = np.asarray(g["number"])
    a["type"] = np.asarray(g["type"])
    a["mass"] = np.asarray(g["mass"], np.float64)
    n = len(a["x"])
    shuffled = np.random.default_rng(3).permutation(n)
    for flags in (7, 6, 5, 3, 1, 0):
        assert s.format_atoms(flags) == _printf_lines(a, flags, range(n)), flags
    assert s.format_atoms(7, shuffled) == _printf_lines(a, 7, shuffled)
    assert s.format_atoms(7, shuffled[:10]) == _printf_lines(a, 7, shuffled[:10])
