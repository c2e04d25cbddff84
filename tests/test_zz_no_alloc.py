"""pmx_dot_noalloc, the dot product for callers that cannot let a library
allocate GPU memory (a JAX process that preallocated the device for its own
pool, or a framework custom call restricted to the framework's allocator).
It keeps its partial sums in a static device array instead of allocating;
this checks it against pmx_dot through the C ABI on two calls in a row (the
array keeps the previous call's contents, which must not leak into the
next result) and that it rejects sizes above its stated maximum."""

import numpy as np
import pytest
import torch

from pmwd_gb300 import _lib

pytestmark = pytest.mark.gpu

RTOL = 1e-12   # float64 sums of float32 products; only the summation order differs


def _dot(name, x, y, n, dev):
    out = torch.full((), float('nan'), dtype=torch.float64, device=dev)
    _lib.call(name, x, y, n, out, _lib.stream_ptr(dev))
    torch.cuda.synchronize(dev)
    return float(out)


def test_noalloc_dot_matches_pmx_dot(cuda):
    g = torch.Generator(device=cuda)
    g.manual_seed(7)
    for n in (3 * 1_000_003, 5, 1 << 17):
        x = torch.randn(n, generator=g, device=cuda)
        y = torch.randn(n, generator=g, device=cuda)
        ref = _dot('pmx_dot', x, y, n, cuda)
        exact = float((x.double() * y.double()).sum())
        assert abs(ref - exact) <= RTOL * max(abs(exact), 1.0) * 10
        for _ in range(2):   # two calls in a row share the static array
            got = _dot('pmx_dot_noalloc', x, y, n, cuda)
            assert abs(got - ref) <= RTOL * max(abs(ref), 1.0), (n, got, ref)


def test_noalloc_dot_rejects_oversize(cuda):
    lib = _lib.load()
    x = torch.zeros(4, device=cuda)
    out = torch.zeros((), dtype=torch.float64, device=cuda)
    st = lib.pmx_dot_noalloc(_lib.ptr(x), _lib.ptr(x), (1 << 30) + 1, _lib.ptr(out),
                             _lib.stream_ptr(cuda))
    assert st == -2
    assert b'maximum' in lib.pmx_last_error()
