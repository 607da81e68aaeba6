"""Index arithmetic of the register unpack of the FP32 z passes
(vonkarman_gb300/csrc/vk_lines.cuh: unpack_rows; vonkarman_gb300/csrc/vk_p3f.cuh:
phase D), checked on the CPU with a model of the last Stockham stage.

Butterfly j (lane j of an NS-lane group) of the last stage of an L = NS * RAD
point forward transform holds Z(k) at k = j + NS r, r < RAD.  The unpack of
mode k needs Z(L - k mod L): the kernels take it from output RAD - 1 - r of
lane (NS - j) mod NS, or, for j = 0, from output (RAD - r) mod RAD of the same
lane.  The unpacked pair must equal the Hermitian split of two real fields
packed as Z = X + i Y, for every kept mode k < H = L / 3 + 1."""

import numpy as np
import pytest

# (NS, RAD) of the forward transforms' last stages on the contiguous FP32 plans:
# 384 = 16 x 24 (k_p3f, k_adj_z at N=256), 768 = 32 x 24 (k_p3 at N=512),
# 192 = 16 x 12, 96 = 16 x 6, 48 = 16 x 3
SHAPES = [(16, 24), (32, 24), (16, 12), (16, 6), (16, 3)]


def lanes_of(z, ns, rad):
    """v[j][r] = Z(j + NS r): the registers of the last stage's butterflies."""
    return np.array([[z[j + ns * r] for r in range(rad)] for j in range(ns)])


def partner(v, j, r, ns, rad):
    if j == 0:
        return v[0][(rad - r) % rad]
    return v[(ns - j) % ns][rad - 1 - r]


@pytest.mark.parametrize("ns,rad", SHAPES)
def test_partner_is_mirror_mode(ns, rad):
    L = ns * rad
    rng = np.random.default_rng(ns * 1000 + rad)
    z = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    v = lanes_of(z, ns, rad)
    for j in range(ns):
        for r in range(rad):
            k = j + ns * r
            assert partner(v, j, r, ns, rad) == z[(L - k) % L], (ns, rad, j, r)


@pytest.mark.parametrize("ns,rad", SHAPES)
def test_register_unpack_equals_hermitian_split(ns, rad):
    L = ns * rad
    H = L // 3 + 1
    rng = np.random.default_rng(7 + ns + rad)
    x, y = rng.standard_normal(L), rng.standard_normal(L)
    z = np.fft.fft(x + 1j * y)
    X, Y = np.fft.fft(x), np.fft.fft(y)
    v = lanes_of(z, ns, rad)
    seen = set()
    for j in range(ns):
        for r in range(rad):
            k = j + ns * r
            if k >= H:
                continue
            zk, w = v[j][r], partner(v, j, r, ns, rad)
            xk = complex(0.5 * (zk.real + w.real), 0.5 * (zk.imag - w.imag))
            yk = complex(0.5 * (zk.imag + w.imag), 0.5 * (w.real - zk.real))
            assert abs(xk - X[k]) < 1e-9 * L and abs(yk - Y[k]) < 1e-9 * L, (ns, rad, k)
            seen.add(k)
    # every kept mode is stored exactly once, and the kernels' loop bound
    # r * NS < H covers them all
    assert seen == set(range(H))
    assert max(r for r in range(rad) if r * ns < H) == (H - 1) // ns


def test_p3f_exchange_index_identities():
    """k_p3f's exchange layouts (vonkarman_gb300/csrc/vk_p3f.cuh): the inverse
    exchange puts position p at p + p // 24 (stride LPA = 408 per line), the
    forward one at p + p // 16 (LPF = 412).  The kernel indexes them with the
    closed forms below; each must equal the layout and stay inside its line."""
    LPA, LPF = 408, 412
    ia = lambda p: p + p // 24
    iff = lambda p: p + p // 16
    for j in range(16):            # phase A writes positions 24 j + r
        for r in range(24):
            assert ia(24 * j + r) == 25 * j + r < LPA
    for jp in range(24):           # phase B reads positions jp + 24 r
        for r in range(16):
            assert ia(jp + 24 * r) == jp + 25 * r < LPA
    for j in range(16):            # phase C reads positions j + 16 r
        for r in range(24):
            assert iff(j + 16 * r) == j + 17 * r < LPF
    # the forward exchange fits inside the inverse one (2 column pairs per CTA)
    assert 6 * LPF <= 12 * LPA
