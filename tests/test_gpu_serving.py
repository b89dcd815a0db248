"""The serving loop on the GPU: every request's result through the server
(mixed stream, overlapping, coalesced) equals its result alone through the
plain entry point and the oracle; budget admission and rejection."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_result(port, spec, src):
    from parallelalgorithms_gb300 import serving
    if spec.op == serving.REQ_SORT:
        return port.sort(src)[0]
    if spec.op == serving.REQ_SELECT:
        return port.select(src, spec.k)
    return np.bincount((src & src.dtype.type(255)).astype(np.int64), minlength=256).astype(np.uint64)


def test_results_same_alone_and_in_the_mix(pa, port, torch_cuda):
    from parallelalgorithms_gb300 import serving
    specs = serving.make_specs(60, seed=11, lo=1e3, hi=3e6)
    bufs = serving.materialize(specs)
    alone, _ = serving.run_plain(specs, bufs)
    alone_sorted = [b[0].copy() if s.op == serving.REQ_SORT else None for s, b in zip(specs, bufs)]
    with serving.Server(max_inflight=4, max_batch_requests=16) as srv:
        reqs = serving.run_served(srv, specs, bufs, rate=None)
        st = srv.stats()
    assert st["completed"] == len(specs) and st["rejected"] == 0
    assert st["batched_units"] >= 1  # waiting requests shared units
    # every kind shared a unit with others of its kind at least once: 32-bit
    # sorts (one segmented launch), 64-bit sorts and selects (one stream),
    # histograms (one launch over all their arrays)
    shared = {(s.op, s.key_kind) for s, r in zip(specs, reqs) if r.c.unit_size > 1}
    assert (serving.REQ_SORT, serving.KEY_U32) in shared and (serving.REQ_SORT, serving.KEY_U64) in shared
    assert any(op == serving.REQ_SELECT for op, _ in shared) and any(op == serving.REQ_HISTOGRAM for op, _ in shared)
    for s, r, a, a_sorted, (buf, _, src) in zip(specs, reqs, alone, alone_sorted, bufs):
        assert r.c.status == 0
        want = _oracle_result(port, s, src)
        if s.op == serving.REQ_SORT:
            np.testing.assert_array_equal(buf, a_sorted)
            np.testing.assert_array_equal(buf, want)
        elif s.op == serving.REQ_SELECT:
            assert int(r.result[0]) == int(a[0]) == want
        else:
            np.testing.assert_array_equal(r.result, a)
            np.testing.assert_array_equal(r.result, want)
        assert r.c.t_submit <= r.c.t_admit <= r.c.t_done


def test_poisson_arrivals_and_device_buffers(pa, port, torch_cuda):
    from parallelalgorithms_gb300 import serving, workloads
    torch = torch_cuda
    specs = serving.make_specs(30, seed=12, lo=1e3, hi=1e6)
    bufs = serving.materialize(specs)
    with serving.Server() as srv:
        reqs = serving.run_served(srv, specs, bufs, rate=2000.0)
        for s, r, (buf, _, src) in zip(specs, reqs, bufs):
            assert r.c.status == 0
            if s.op == serving.REQ_SORT:
                np.testing.assert_array_equal(buf, np.sort(src))
        # device-resident keys are sorted in place
        a = workloads.uniform_u32(500_000, seed=3)
        d = torch.from_numpy(a.view(np.int32).copy()).cuda()
        r = serving.Request(serving.REQ_SORT, d)
        srv.submit(r)
        assert srv.wait(r) == 0
        np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), np.sort(a))


def test_budget_admission_and_rejection(pa, torch_cuda):
    from parallelalgorithms_gb300 import serving, workloads
    budget = 64 << 20  # 64 MiB
    with serving.Server(budget_bytes=budget, max_inflight=8, coalesce=False) as srv:
        small = [serving.Request(serving.REQ_SORT, workloads.uniform_u32(1_000_000, seed=i)) for i in range(6)]
        big = serving.Request(serving.REQ_SORT, workloads.uniform_u64(20_000_000, seed=9))  # ~330 MB: never fits
        for r in small:
            srv.submit(r)
        srv.submit(big)
        srv.drain()
        st = srv.stats()
    assert all(r.c.status == 0 for r in small)
    assert big.c.status == 2  # PA_ERR_OOM: larger than the whole budget
    assert st["rejected"] == 1 and st["peak_bytes"] <= budget
    for r in small:
        k = r.keys
        assert np.all(k[1:] >= k[:-1])


def test_join_limits(pa, port, torch_cuda):
    """Requests above the join limit run alone; invalid limits are refused."""
    from parallelalgorithms_gb300 import serving
    with pytest.raises(pa.PaError):
        serving.Server(join_max_keys_log2=41)
    with pytest.raises(pa.PaError):
        serving.Server(unit_max_keys_log2=-1)
    specs = serving.make_specs(40, seed=13, lo=1e2, hi=1e5)
    bufs = serving.materialize(specs)
    with serving.Server(max_inflight=2, join_max_keys_log2=10, unit_max_keys_log2=12) as srv:
        reqs = serving.run_served(srv, specs, bufs, rate=None)
        st = srv.stats()
    assert st["completed"] == len(specs)
    for s, r, (buf, _, src) in zip(specs, reqs, bufs):
        assert r.c.status == 0
        if s.n > 1024:
            assert r.c.unit_size == 1
        if s.op == serving.REQ_SORT:
            np.testing.assert_array_equal(buf, port.sort(src)[0])
