"""Batched segmented sort vs the oracle, bit-exact per segment, through the
C ABI (plans replayed from a CUDA graph, the one-shot form, every tuning
configuration, the autotuner)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_segments(sizes, seed=1238):
    from parallelalgorithms_gb300 import workloads
    sizes = np.asarray(sizes, dtype=np.uint64)
    off = np.zeros(sizes.size + 1, np.uint64)
    off[1:] = np.cumsum(sizes)
    keys = workloads.uniform_u32(int(off[-1]), seed=seed)
    # a few segments with heavy ties and presorted runs
    rng = np.random.default_rng(seed)
    for i in range(0, sizes.size, 7):
        a, b = int(off[i]), int(off[i + 1])
        keys[a:b] = rng.integers(0, 5, b - a, dtype=np.uint32)
    for i in range(3, sizes.size, 11):
        a, b = int(off[i]), int(off[i + 1])
        keys[a:b] = np.arange(b - a, dtype=np.uint32)
    return keys, off


def edge_sizes():
    s = [0, 1, 2, 3, 17, 100, 2047, 2048, 2049, 4095, 4096, 4097, 8191, 8192, 8193, 16384, 65537, 200003]
    rng = np.random.default_rng(7)
    s += list(np.round(np.exp(rng.uniform(np.log(1e3), np.log(3e5), 150))).astype(int))
    return s


def check(port, keys, out, off):
    for i in range(off.size - 1):
        a, b = int(off[i]), int(off[i + 1])
        want, _ = port.sort(keys[a:b])
        np.testing.assert_array_equal(out[a:b], want, err_msg=f"segment {i} [{a}, {b})")


@pytest.mark.parametrize("cutoff", [2048, 4096, 8192])
@pytest.mark.parametrize("tile", [4096, 8192])
@pytest.mark.parametrize("bits", [8, 11])
def test_plan_every_config_matches_oracle(pa, port, torch_cuda, cutoff, tile, bits):
    """8-bit digits (four passes) and 11-bit digits (three passes of the
    2048-bin tile, the result copied back from the scratch buffer)."""
    from parallelalgorithms_gb300.batched import SegmentedSortPlan, SegSortChoice
    torch = torch_cuda
    keys, off = make_segments(edge_sizes())
    plan = SegmentedSortPlan(off, SegSortChoice(cutoff, tile, bits), use_graph=True)
    info = plan.info()
    assert info["small_segments"] > 0 and info["large_segments"] > 0
    d = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    t = torch.empty_like(d)
    for _ in range(2):  # second run replays the captured graph
        d.copy_(torch.from_numpy(keys.view(np.int32)))
        plan.run(d, t)
        check(port, keys, d.cpu().numpy().view(np.uint32), off)
    # a different buffer re-captures the graph
    d2 = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    plan.run(d2, t)
    check(port, keys, d2.cpu().numpy().view(np.uint32), off)
    plan.close()


def test_one_shot_host_and_device(pa, port, torch_cuda):
    from parallelalgorithms_gb300.batched import segmented_sort
    keys, off = make_segments(edge_sizes()[:60], seed=99)
    h = keys.copy()
    segmented_sort(h, off)
    check(port, keys, h, off)
    d = torch_cuda.from_numpy(keys.view(np.int32).copy()).cuda()
    segmented_sort(d, off)
    check(port, keys, d.cpu().numpy().view(np.uint32), off)


def test_async_runs_and_autotuner(pa, port, torch_cuda, tmp_path, monkeypatch):
    from parallelalgorithms_gb300 import batched
    monkeypatch.setenv("PA_AUTOTUNE_FILE", str(tmp_path / "tune.json"))
    torch = torch_cuda
    keys, off = make_segments(edge_sizes()[:80], seed=5)
    d = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    t = torch.empty_like(d)
    res = batched.autotune(off, d, t, reps=1)
    assert res["choice"] in batched.CANDIDATES and len(res["ms"]) == len(batched.CANDIDATES)
    assert batched.load_choice(off) == res["choice"]
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), keys)  # autotune restores the input
    plan = batched.SegmentedSortPlan(off, batched.load_choice(off))
    stream = torch.cuda.current_stream().cuda_stream
    plan.run(d, t, stream, sync=False)
    plan.sync(stream)
    check(port, keys, d.cpu().numpy().view(np.uint32), off)


def test_empty_and_degenerate_segmentations(pa, torch_cuda):
    from parallelalgorithms_gb300.batched import SegmentedSortPlan
    plan = SegmentedSortPlan(np.zeros(5, np.uint64))  # four empty segments
    assert plan.info()["work_items"] == 0
    d = torch_cuda.zeros(1, dtype=torch_cuda.int32, device="cuda")
    plan.run(d, d)
    with pytest.raises(pa.PaError):
        SegmentedSortPlan(np.array([0, 10, 5], np.uint64))  # decreasing offsets
