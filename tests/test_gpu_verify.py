"""The device-side verifier (librett_c_verify) and full-size checks with it.

The verifier itself is checked against the oracle first: zero mismatches on
correct outputs of several shapes, and exactly the planted mismatches (made
by flipping bytes of a correct output) at the right first index.  Then it
checks every element of the full-size small-leading-dimension problems
(4 GB and 503 MB each way), which are too large for the host oracle.
"""
import numpy as np
import pytest

import librett_gb300 as L
from oracle import oracle as O
from tests import shapes as S

pytestmark = pytest.mark.gpu

SMALL = [S.C1, (S.EXAMPLE[0], S.EXAMPLE[1], 16), ([37, 5, 41, 3], [2, 0, 3, 1], 8),
         ([3] * 16, list(range(15, -1, -1)), 4), ([1000, 3, 7], [0, 2, 1], 8),
         ([5, 7], [0, 1], 4)]


def _transpose(dims, perm, es, host):
    import torch

    inp = torch.from_numpy(host).cuda()
    out = torch.zeros_like(inp)
    with L.Plan(dims, perm, es, torch.cuda.current_stream()) as p:
        p.execute(inp.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    return inp, out


@pytest.mark.parametrize("dims,perm,es", SMALL)
def test_verifier_against_oracle(cuda, dims, perm, es):
    import torch

    vol = int(np.prod(dims))
    host = np.random.default_rng(vol).integers(0, 256, vol * es, dtype=np.uint8)
    inp, out = _transpose(dims, perm, es, host)
    assert np.array_equal(out.cpu().numpy(), O.transpose_np(host, dims, perm, es).view(np.uint8))
    s = torch.cuda.current_stream()
    assert L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), s) == (0, -1)
    # plant mismatches in a correct output: one byte of element k, and (when
    # there is room) one byte of a later element
    k = vol // 3
    out[k * es + es - 1] ^= 0x01
    assert L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), s) == (1, k)
    if vol > k + 2:
        out[(vol - 1) * es] ^= 0x80
        assert L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), s) == (2, k)


def test_verifier_rejects_bad_arguments(cuda):
    import torch

    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(L.LibrettError):
        L.verify([4, 4], [0, 0], 4, buf.data_ptr(), buf.data_ptr())
    with pytest.raises(L.LibrettError):
        L.verify([4, 4], [1, 0], 4, buf.data_ptr() + 2, buf.data_ptr())


@pytest.mark.parametrize("dims,perm,es", [S.C3A, S.C3B])
def test_full_size_small_leading_dims_every_element(cuda, dims, perm, es):
    import torch

    vol = int(np.prod(dims))
    g = torch.Generator(device="cuda")
    g.manual_seed(vol % 1000003)
    inp = torch.randint(-(2 ** 62), 2 ** 62, ((vol * es + 7) // 8,), dtype=torch.int64,
                        device="cuda", generator=g).view(torch.uint8)[:vol * es]
    out = torch.zeros_like(inp)
    s = torch.cuda.current_stream()
    with L.Plan(dims, perm, es, s) as p:
        p.execute(inp.data_ptr(), out.data_ptr())
    assert L.verify(dims, perm, es, inp.data_ptr(), out.data_ptr(), s) == (0, -1)
