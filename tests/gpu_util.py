"""Helpers for GPU tests: column-major transfers between numpy and CUDA tensors."""
import numpy as np
import torch


def to_dev(X, device="cuda:0"):
    """numpy (M, N) -> CUDA tensor (M, N) stored column-major (stride (1, M))."""
    X = np.asarray(X)
    return torch.from_numpy(np.ascontiguousarray(X.T)).to(device).t()


def to_dev_ld(X, ld, fill=np.nan, device="cuda:0"):
    """Column-major CUDA view of X inside a larger buffer with leading dimension ld."""
    M, N = X.shape
    buf = np.full((ld, max(N, 1)), fill, dtype=X.dtype)
    buf[:M, :N] = X
    t = to_dev(buf, device)
    return t[:M, :N], t


def to_host(T):
    """CUDA tensor (any strides) -> numpy (M, N) Fortran-ordered copy."""
    return np.asfortranarray(T.detach().cpu().numpy())


def bits(x):
    x = np.asarray(x)
    return x.view(np.uint64 if x.dtype == np.float64 else np.uint32)


def assert_bit_equal(got, ref):
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape and got.dtype == ref.dtype
    if got.dtype.kind in "iu":
        bad = got != ref
        if bad.any():
            idx = np.argwhere(bad)[:5]
            raise AssertionError("%d mismatches, e.g. %s: got %r ref %r" % (
                bad.sum(), idx.tolist(), [got[tuple(i)] for i in idx], [ref[tuple(i)] for i in idx]))
        return
    nan_g, nan_r = np.isnan(got), np.isnan(ref)
    assert np.array_equal(nan_g, nan_r), "NaN positions differ"
    ok = nan_g | (bits(got) == bits(ref))
    if not ok.all():
        idx = np.argwhere(~ok)[:5]
        raise AssertionError("%d mismatches, e.g. %s: got %r ref %r" % (
            (~ok).sum(), idx.tolist(), [got[tuple(i)] for i in idx], [ref[tuple(i)] for i in idx]))
