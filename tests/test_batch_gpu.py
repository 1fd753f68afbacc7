"""Batched and served FP32 form through the batch C ABI.

* A scenario's result is the same alone and in a mix of other scenarios of
  different sizes (bit-identical: every tile and every per-scenario
  reduction is independent of the rest of the batch).
* Admission respects the HBM budget and the queue drains as scenarios finish.
* A batch scenario equals the same scenario run through a single FP32 handle.
* Cancelling a running request frees its slot for a queued one and leaves
  the other requests' results unchanged.
"""
import numpy as np
import pytest

from sw2d_efdc_gb300 import api, synth

pytestmark = pytest.mark.gpu


def scenario(side, seed, t_end=120.0):
    rng = np.random.default_rng(seed)
    sc = synth.batch_scenario(side, rng, dx=1.0)
    return dict(dem=sc.dem, manning_classes=sc.manning_classes, manning_table=sc.manning_table,
                rain_mm=sc.rain_mm * 20.0, dtrain=sc.dtrain, dx=1.0, t_end=t_end, outflow=api.OUTFLOW_SOUTH)


def run_batch(specs, budget=0.0, chunk=32):
    b = api.Batch(hbm_budget_bytes=budget)
    ids = [b.submit(**s) for s in specs]
    for _ in range(10000):
        nr, nq = b.step(chunk)
        if nr == 0 and nq == 0:
            break
    out = {}
    for i in ids:
        st, led = b.poll(i)
        assert st == api.REQ_DONE, st
        out[i] = (b.result(i), led)
    stats = b.stats()
    b.close()
    return [out[i] for i in ids], stats


def test_same_alone_and_in_the_mix():
    a = scenario(150, 1)
    (alone,), _ = run_batch([a])
    mix, stats = run_batch([scenario(200, 2, 90.0), a, scenario(97, 3, 60.0), scenario(260, 4, 150.0)])
    (h0, qx0, qy0), l0 = alone
    (h1, qx1, qy1), l1 = mix[1]
    assert np.array_equal(h0, h1) and np.array_equal(qx0, qx1) and np.array_equal(qy0, qy1)
    assert l0["iterations"] == l1["iterations"] and l0["time"] == l1["time"] == 120.0
    assert stats["cell_updates"] > 0


def test_budget_admission_and_drain():
    specs = [scenario(128, 10 + k, 40.0) for k in range(5)]
    # one 128 x 128 scenario holds about 0.72 MB (33 B per padded cell of
    # 160 x 136); this budget has room for two at a time
    b = api.Batch(hbm_budget_bytes=2.5 * 128 * 136 * 40)
    ids = [b.submit(**s) for s in specs]
    nr, nq = b.step(0)
    assert nr == 2 and nq == 3
    seen_running = []
    for _ in range(10000):
        nr, nq = b.step(16)
        seen_running.append(nr)
        if nr == 0 and nq == 0:
            break
    assert max(seen_running) <= 2
    for i in ids:
        assert b.poll(i)[0] == api.REQ_DONE
    with pytest.raises(api.Sw2dError):
        b.submit(**scenario(1024, 99))  # larger than the whole budget
    b.close()


def test_batch_equals_single_fp32_handle():
    s = scenario(130, 7, 80.0)
    (res,), _ = run_batch([s])
    cfg = api.default_config(rows=130, cols=130, precision=api.FP32, dt_mode=api.DT_CFL,
                             series_mode=api.SERIES_STEP, dx=1.0, dy=1.0, cfl=0.7, dt_max=2.0,
                             outflow=api.OUTFLOW_SOUTH)
    m = api.Model(cfg)
    m.set_dem(s["dem"])
    m.set_manning_classes(s["manning_classes"], s["manning_table"])
    m.set_rain_series(s["rain_mm"], s["dtrain"])
    m.set_depth(np.zeros_like(s["dem"]))
    m.advance(80.0)
    h, qx, qy = m.state()
    assert np.array_equal(h, res[0][0]) and np.array_equal(qx, res[0][1])


def test_cancel_mid_run_frees_the_slot_and_leaves_the_others_unchanged():
    """Releasing a running request cancels it between steps: its memory goes
    back to the budget, a queued request is admitted in its place, and the
    other requests finish exactly as they would alone."""
    a, b_, c = scenario(128, 21, 60.0), scenario(128, 22, 60.0), scenario(128, 23, 60.0)
    alone = {k: run_batch([s])[0][0] for k, s in (("a", a), ("c", c))}
    bt = api.Batch(hbm_budget_bytes=2.5 * 128 * 136 * 40)
    ia, ib, ic = (bt.submit(**s) for s in (a, b_, c))
    nr, nq = bt.step(8)
    assert (nr, nq) == (2, 1)
    assert bt.poll(ib)[0] == api.REQ_RUNNING
    bt.release(ib)
    with pytest.raises(api.Sw2dError) as e:
        bt.poll(ib)
    assert e.value.code == api.SW2D_ERR_NOT_FOUND
    for _ in range(10000):
        nr, nq = bt.step(32)
        if nr == 0 and nq == 0:
            break
    for k, i in (("a", ia), ("c", ic)):
        st, led = bt.poll(i)
        assert st == api.REQ_DONE
        (h0, qx0, qy0), l0 = alone[k]
        h1, qx1, qy1 = bt.result(i)
        assert np.array_equal(h0, h1) and np.array_equal(qx0, qx1) and np.array_equal(qy0, qy1)
        assert led["time"] == l0["time"] == 60.0
    bt.close()


def test_rows_per_item_does_not_change_results():
    """The rows per work item and the CTAs per SM (the autotuner's knobs)
    change only the work split: the bed's datum tiles are fixed at 224 x 64
    cells, so every setting, and the tuned default, gives bit-identical
    results, alone and in a mix."""
    a = scenario(300, 31, 60.0)

    def run(specs, rows):
        b = api.Batch()
        b.set_rows_per_item(rows)
        ids = [b.submit(**s) for s in specs]
        while b.step(32) != (0, 0):
            pass
        out = b.result(ids[-1])
        st = b.stats()
        b.close()
        return out, st

    ref, st = run([a], 256)
    assert st["rows_per_item"] == 256
    for rows, specs in ((64, [a]), (128, [scenario(500, 32, 30.0), scenario(140, 33, 90.0), a]), (512, [a]),
                        (0, [scenario(1200, 34, 20.0), a])):
        got, st = run(specs, rows)
        assert all(np.array_equal(x, y) for x, y in zip(ref, got)), rows
        if rows == 0:  # 1.53 M cells: the autotuner timed one size bucket
            assert st["tunings"] == 1 and st["rows_per_item"] in (64, 128, 256, 512)
            assert st["ctas_per_sm"] >= 0
    b = api.Batch()
    with pytest.raises(api.Sw2dError):
        b.set_rows_per_item(30)
    with pytest.raises(api.Sw2dError):
        b.set_rows_per_item(1024)
    b.close()


def test_explicit_tuning_runs_once_per_size_bucket():
    """sw2d_batch_tune times every candidate work split on the scenarios' own
    iterations before any step (so a caller keeps it out of the steps it
    times), caches the choice for the size bucket, counts its iterations in
    neither the device time nor the cell-updates, and leaves the results
    bit-identical to a fixed split."""
    specs = [scenario(1100, 51, 40.0), scenario(300, 52, 60.0)]
    b = api.Batch()
    b.set_rows_per_item(256)
    ids = [b.submit(**s) for s in specs]
    assert b.tune(264) == 0  # rows per item fixed: nothing to tune
    while b.step(32) != (0, 0):
        pass
    ref = [b.result(i) for i in ids]
    b.close()
    b = api.Batch()
    ids = [b.submit(**s) for s in specs]
    assert b.tune(11) == 0  # too few iterations: fewer than three per candidate
    n = b.tune(264)
    assert n == 264  # eight candidates (four CTAs per SM fit) x (1 untimed + 32 timed)
    assert b.tune(264) == 0  # the bucket is cached
    st = b.stats()
    assert st["tunings"] == 1 and st["tuning_iterations"] == n
    assert st["device_ms"] == 0.0 and st["cell_updates"] == 0.0
    assert st["rows_per_item"] in (64, 128, 256, 512) and st["ctas_per_sm"] >= 0
    while b.step(32) != (0, 0):
        pass
    got = [b.result(i) for i in ids]
    b.close()
    for x, y in zip(ref, got):
        assert all(np.array_equal(p, q) for p, q in zip(x, y))


def test_request_submitted_while_others_run_matches_alone():
    """Continuous batching: a request that arrives while other requests are
    already advancing on the GPU joins at the next step and finishes
    bit-identical to the same request run alone; the requests that were
    running are unchanged by its arrival."""
    late = scenario(170, 41, 70.0)
    early = [scenario(240, 42, 90.0), scenario(120, 43, 50.0)]
    alone_late = run_batch([late])[0][0]
    alone_early = [run_batch([s])[0][0] for s in early]
    b = api.Batch()
    ids = [b.submit(**s) for s in early]
    nr, nq = b.step(24)
    assert nr == 2 and nq == 0
    assert all(b.poll(i)[0] == api.REQ_RUNNING for i in ids)
    t_before = [b.poll(i)[1]["time"] for i in ids]
    assert all(0.0 < t < 50.0 for t in t_before)  # mid-run
    il = b.submit(**late)
    nr, nq = b.step(8)
    assert nr == 3 and b.poll(il)[0] == api.REQ_RUNNING
    for _ in range(10000):
        nr, nq = b.step(32)
        if nr == 0 and nq == 0:
            break
    for i, (res, led) in zip(ids + [il], alone_early + [alone_late]):
        st, l1 = b.poll(i)
        assert st == api.REQ_DONE
        got = b.result(i)
        assert all(np.array_equal(x, y) for x, y in zip(got, res))
        assert l1["time"] == led["time"] and l1["iterations"] == led["iterations"]
    b.close()
