"""Precision of pass 1's twiddle generation, restated on the CPU in float32.

k_twiddle_sum (cuspfft_gb300/csrc/gbsp_kernels.cuh, column_sums_warp) gives
each lane the Bluestein rows u, u+32, ..., u+224 of a nonzero r.  Per group
of four rows it reads W^p exactly from the FP64-built table, forms
n1 = w0 * (-z) with z = W^{(32 r) mod rows}, then n2 = c2*n1 + w0 and
w3 = (-c2)*n2 + n1 with c2 = 2 cos(arg z) (packed FMAs); n1 and n2 are the
negated rows u+32 and u+64 of the group.  These tests restate that sequence
with numpy float32 (an FMA as an exact float64 product plus one rounding)
and check:
  - every twiddle is within 1e-6 of the exact value (the table entries are
    correctly rounded; three recurrence steps at most separate a twiddle from one);
  - the negated carry is bitwise the negative of the plain recurrence
    w[k+1] = c2*w[k] - w[k-1], the form the kernel had before packing;
  - column sums built from these twiddles stay within rel-L2 1e-6 of FP64.
"""
import numpy as np
import pytest

F32 = np.float32


def _fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(F32)


def _cmul(a, b):
    (ar, ai), (br, bi) = a, b
    return _fma(ar, br, -(ai * bi).astype(F32)), _fma(ar, bi, (ai * br).astype(F32))


def _table(p, rows):
    ang = -2.0 * np.pi * p.astype(np.float64) / rows
    return np.cos(ang).astype(F32), np.sin(ang).astype(F32)


def kernel_twiddles(u, r, rows, ku=8):
    """Twiddles W^{(u + 32 k) r}, k < ku, as the kernel forms them."""
    z = _table((32 * r) % rows, rows)
    nz = (-z[0], -z[1])
    c2 = (F32(-2.0) * nz[0]).astype(F32)
    out = []
    for g in range(0, ku, 4):
        w0 = _table(((u + 32 * g) * r) % rows, rows)
        n1 = _cmul(w0, nz)
        n2 = (_fma(c2, n1[0], w0[0]), _fma(c2, n1[1], w0[1]))
        w3 = (_fma(-c2, n2[0], n1[0]), _fma(-c2, n2[1], n1[1]))
        out += [w0, (-n1[0], -n1[1]), (-n2[0], -n2[1]), w3]
    return out


def plain_recurrence(u, r, rows, ku=8):
    """The unpacked form: w1 = w0 * z, w[k+1] = c2 * w[k] - w[k-1]."""
    z = _table((32 * r) % rows, rows)
    c2 = (F32(2.0) * z[0]).astype(F32)
    out = []
    for g in range(0, ku, 4):
        w0 = _table(((u + 32 * g) * r) % rows, rows)
        w1 = _cmul(w0, z)
        w2 = (_fma(c2, w1[0], -w0[0]), _fma(c2, w1[1], -w0[1]))
        w3 = (_fma(c2, w2[0], -w1[0]), _fma(c2, w2[1], -w1[1]))
        out += [w0, w1, w2, w3]
    return out


def _exact(u, r, rows, k):
    return np.exp(-2j * np.pi * (((u + 32 * k) * r) % rows) / rows)


@pytest.mark.parametrize("rows", [97, 3001, 8219, 16706, 40421])
def test_twiddle_error_bound(rows):
    g = np.random.default_rng(rows)
    u = g.integers(0, rows, 50000)
    r = g.integers(0, rows, 50000)
    tw = kernel_twiddles(u, r, rows)
    worst = max(np.max(np.abs(w[0] + 1j * w[1].astype(np.float64) - _exact(u, r, rows, k)))
                for k, w in enumerate(tw))
    assert worst < 1e-6, f"rows={rows}: worst twiddle error {worst:.3e}"


@pytest.mark.parametrize("rows", [3001, 8219])
def test_negated_carry_is_bitwise_the_plain_recurrence(rows):
    g = np.random.default_rng(rows + 1)
    u = g.integers(0, rows, 20000)
    r = g.integers(0, rows, 20000)
    for a, b in zip(kernel_twiddles(u, r, rows), plain_recurrence(u, r, rows)):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_column_sums_against_fp64():
    rows = 8219
    g = np.random.default_rng(5)
    col = np.unique(g.integers(0, rows, 400))          # one column's nonzero rows
    u = np.arange(0, 256)                              # one row block (32 lanes x 8)
    lanes, ks = u % 32, u // 32
    got = np.zeros(u.size, np.complex128)
    for rr in col:
        tw = kernel_twiddles(lanes, np.full(lanes.size, rr), rows)
        got += np.array([tw[k][0][i] + 1j * np.float64(tw[k][1][i]) for i, k in enumerate(ks)])
    want = np.exp(-2j * np.pi * (np.outer(u, col) % rows) / rows).sum(axis=1)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 1e-6, f"rel-L2 {err:.3e}"
