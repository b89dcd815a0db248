"""The 32-bit sort's first digit pass with prepared offsets: the histogram
kernel also writes, per first-pass tile, the keys of each byte-0 value in
the earlier tiles of its chunk and per chunk those of the earlier chunks,
and the first pass reads its tile's two rows instead of looking back.
Sizes sit on the chunk arithmetic's edges (one tile per chunk, a last chunk
of one short tile, several tiles per chunk with a short last tile), checked
bit-exact against the oracle on device buffers, for distributions that run
or skip the first pass, float keys, and a buffer that is not 16-byte
aligned (the plain histogram and look-back instead)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILE = 6144  # first-pass tile of the 32-bit keys-only sort


def _sms(torch):
    return torch.cuda.get_device_properties(0).multi_processor_count


def _sizes(sms):
    return [8193, 2 * TILE, sms * TILE, sms * TILE + 1, 2 * sms * TILE + 6143, 3 * sms * TILE + 5000,
            1_000_003, 7_777_777]


def _inputs(n):
    from parallelalgorithms_gb300 import workloads
    rng = np.random.default_rng(n + 7)
    u = workloads.uniform_u32(n)
    return {
        "uniform": u,
        "byte0_skewed": (u & np.uint32(0xFFFFFF00)) | rng.choice(np.array([0, 1, 2, 255], np.uint32), n,
                                                                   p=[0.7, 0.2, 0.09, 0.01]),
        "byte0_constant": (u & np.uint32(0xFFFFFF00)) | np.uint32(0x5A),  # the first pass is skipped
        "presorted": np.arange(n, dtype=np.uint32),
        "constant": np.full(n, 7, np.uint32),
    }


def _to_dev(torch, a):
    return torch.from_numpy(a.view(np.int32).copy()).cuda()


@pytest.mark.parametrize("k", range(8))
def test_prepared_first_pass_matches_oracle(pa, port, torch_cuda, k):
    n = _sizes(_sms(torch_cuda))[k]
    for name, a in _inputs(n).items():
        want, _ = port.sort(a)
        d = _to_dev(torch_cuda, a)
        pa.sort(d)
        np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), want, err_msg=f"{name} n={n}")


@pytest.mark.parametrize("k", [0, 3, 6])
def test_prepared_first_pass_float_keys(pa, port, torch_cuda, k):
    from parallelalgorithms_gb300 import workloads
    n = _sizes(_sms(torch_cuda))[k]
    a = workloads.normal_specials_f32(n)
    want, _ = port.sort(a)
    d = torch_cuda.from_numpy(a.copy()).cuda()
    pa.sort(d)
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_unaligned_buffer_takes_the_look_back(pa, port, torch_cuda):
    n = _sms(torch_cuda) * TILE + 1
    a = _inputs(n + 1)["uniform"]
    want, _ = port.sort(a[1:])
    base = _to_dev(torch_cuda, a)
    view = base[1:]
    pa.sort(view)
    np.testing.assert_array_equal(view.cpu().numpy().view(np.uint32), want)


def test_repeated_sorts_of_different_sizes(pa, port, torch_cuda):
    """The tables and the chunk ticket are reset by every call (the
    workspace is reused across sizes, larger then smaller)."""
    from parallelalgorithms_gb300 import workloads
    for n in (3 * _sms(torch_cuda) * TILE + 5000, 2 * TILE, 1_000_003, 2 * TILE):
        a = workloads.uniform_u32(n, seed=n)
        want, _ = port.sort(a)
        d = _to_dev(torch_cuda, a)
        pa.sort(d)
        np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), want, err_msg=f"n={n}")
