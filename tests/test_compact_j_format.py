"""The 6-byte copy of L^-1 B that the mixed-path J column sums read
(k_encode_f32i16): per element the FP32 value of its sign, exponent and top
24 significand bits, and the next 29 bits rounded to a 16-bit integer
(min(rint(m29 / 2^13), 65535)).  Restated here in numpy: every element keeps
a relative error below 2^-39, and J computed from the copy stays within
1e-11 of J from the FP64 tensor on butane (the device test bar for the mixed
J is 1e-9)."""
import numpy as np


def encode_decode(x):
    """x (FP64) -> the value the compact copy represents, as FP64."""
    u = np.ascontiguousarray(x, np.float64).view(np.uint64)
    E = ((u >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    ef = E - 896  # FP32 biased exponent of the top part
    hi = (u & ~np.uint64((1 << 29) - 1)).view(np.float64)
    m29 = (u & np.uint64((1 << 29) - 1)).astype(np.int64)
    lo16 = np.minimum((m29 + 4096) >> 13, 65535)
    sign = np.where(x < 0, -1.0, 1.0)
    lo = sign * lo16.astype(np.float64) * np.exp2((E - 1062).astype(np.float64))
    ok = (ef >= 1) & (ef <= 254)
    # the remainder's scale 2^(ef - 39 - 127) must itself be an FP32 normal
    lo = np.where(ef - 39 >= 1, lo, 0.0)
    return np.where(ok, hi + lo, 0.0)


def test_element_precision():
    rng = np.random.default_rng(5)
    x = rng.standard_normal(200000) * np.exp2(rng.integers(-40, 20, 200000))
    y = encode_decode(x)
    rel = np.abs(y - x) / np.abs(x)
    assert rel.max() < 2.0 ** -39
    # values beyond the FP32 normal range are dropped, as in the kernel
    assert np.all(encode_decode(np.array([1e-40, -1e300])) == 0.0)


def test_j_from_the_compact_copy(butane):
    ds = butane
    lay = ds.layout
    sv, U = np.linalg.eigh(ds.S)
    X = U @ np.diag(sv ** -0.5) @ U.T
    _, Cp = np.linalg.eigh(X.T @ ds.Hcore @ X)
    C = (X @ Cp)[:, :ds.nocc]
    P = 2.0 * C @ C.T
    LB = np.einsum("yx,xmn->ymn", np.tril(ds.Linv), lay.to_dense(ds.B), optimize=True)
    d = np.einsum("ymn,mn->y", LB, P)
    J = np.einsum("y,ymn->mn", d, LB)
    Jc = np.einsum("y,ymn->mn", d, encode_decode(LB).reshape(LB.shape))
    assert np.abs(Jc - J).max() <= 1e-11
    assert abs(0.5 * np.sum(P * (Jc - J))) <= 1e-9
