"""CPU tests of host-side logic around the GPU path (no device needed).

* the panel schedule the bench's algorithmic counts follow (the factor's own rule:
  nb-wide panels, then nb/2-wide ones for the last OOC_OPT_TAIL_ORDER orders of a
  split-BF16 factor whose nb is a multiple of 256);
* the batched autotuner's JSON table: save, merge per GPU and precision, load back,
  unreadable files;
* the served request trace: arrival rate, repeat share, order distribution, repeats
  naming earlier matrices, determinism;
* the clock record taken during the timed region: median SM clock, maximum, and the
  throttle reasons a measurement is judged by;
* the CPU path's single-request times that the serving report carries.
"""
import json
import math
import os

import pytest

import bench
from oocdag_gb300 import autotune


# ---------------------------------------------------------------- panel schedule
def _check_cover(panels, n):
    J = 0
    for J0, w in panels:
        assert J0 == J and w > 0
        J += w
    assert J == n


@pytest.mark.parametrize("n,nb,prec,tail", [(65536, 512, "bf16x3", 24576), (600, 256, "bf16x3", 24576),
                                            (1000, 512, "bf16x3", 600), (32768, 256, "bf16x3", 0),
                                            (65536, 512, "fp32", 24576), (1001, 384, "bf16x3", 500)])
def test_panel_schedule_covers_the_matrix(n, nb, prec, tail):
    P = bench.panel_schedule(n, nb, prec, tail)
    _check_cover(P, n)
    split = prec == "bf16x3" and nb % 256 == 0 and n > nb and tail > 0
    t0 = n
    if split:
        t0 = min(n, -(-max(0, n - tail) // nb) * nb)
    for J0, w in P:
        if J0 < t0:
            assert w == min(nb, n - J0)
        else:
            assert split and w == min(nb // 2, n - J0)


def test_panel_schedule_default_workload():
    P = bench.panel_schedule(65536, 512, "bf16x3", 24576)
    assert len(P) == 176
    assert sum(1 for _, w in P if w == 512) == 80 and sum(1 for _, w in P if w == 256) == 96
    assert P[80] == (40960, 256)


# ---------------------------------------------------------------- autotuner table
@pytest.mark.parametrize("n,block_cols", [(65536, -1), (16384, -1), (20000, 2048), (65536, 0)])
def test_update_schedule_accounts_for_the_cholesky_flops(n, block_cols):
    # The bench's roofline counts 2 K flops per lower-triangle output element of every
    # trailing-update launch in the schedule the library runs (left-looking catch-ups and
    # in-block updates, or right-looking panels).  Together they must be the Cholesky's
    # n^3/3 less the diagonal tiles' own factor and column-solve work: never more, and
    # only a small share less.
    nb = 512
    s = bench.update_schedule(n, nb, "bf16x3", 24576, block_cols)
    upd = sum(2 * K * bench.lower_elems(m, c) for m, K, c in s["launches"])
    total = n ** 3 / 3
    diag = sum(LN ** 3 / 3 + (n - J0 - LN) * LN * LN for J0, LN in s["panels"])
    assert upd <= total
    assert abs(upd + diag - total) <= 0.01 * total, (upd, diag, total)
    if block_cols != 0:
        assert s["kind"].startswith("left-looking")
        assert all(K <= bench.CATCH_K for _, K, _ in s["launches"])


def test_autotune_table_round_trip(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "_gpu_name", lambda: "Test GPU")
    path = str(tmp_path / "sub" / "t.json")
    r64 = {"gpu": "Test GPU", "prec": "fp64", "table": [32] * 16}
    r32 = {"gpu": "Test GPU", "prec": "fp32", "table": [64] * 16}
    other = {"gpu": "Other GPU", "prec": "fp64", "table": [8] * 16}
    assert autotune.load_table("fp64", path) is None
    assert autotune.save(r64, path) == path
    autotune.save(r32, path)
    autotune.save(other, path)
    assert autotune.load_table("fp64", path) == [32] * 16
    assert autotune.load_table("fp32", path) == [64] * 16
    data = json.load(open(path))
    assert set(data) == {"Test GPU|fp64", "Test GPU|fp32", "Other GPU|fp64"}
    assert not os.path.exists(path + ".tmp")
    r64b = dict(r64, table=[16] * 16)  # a re-tune replaces the entry
    autotune.save(r64b, path)
    assert autotune.load_table("fp64", path) == [16] * 16


def test_autotune_unreadable_table(tmp_path, monkeypatch):
    monkeypatch.setattr(autotune, "_gpu_name", lambda: "Test GPU")
    path = str(tmp_path / "t.json")
    open(path, "w").write("{not json")
    assert autotune.load_table("fp64", path) is None
    autotune.save({"gpu": "Test GPU", "prec": "fp64", "table": [32] * 16}, path)
    assert autotune.load_table("fp64", path) == [32] * 16


# ---------------------------------------------------------------- served trace
def test_request_trace_statistics():
    rate, seconds = 200, 10.0
    tr = bench.make_trace(rate, seconds, seed=7)
    k = len(tr)
    assert abs(k - rate * seconds) < 5 * math.sqrt(rate * seconds)
    ts = [r["t"] for r in tr]
    assert ts == sorted(ts) and 0 < ts[0] and ts[-1] <= seconds
    new = [r for r in tr if r["kind"] == 0]
    rep = [r for r in tr if r["kind"] == 1]
    assert abs(len(rep) / k - 0.3) < 0.05
    assert [r["key"] for r in new] == list(range(1, len(new) + 1))
    big = [r for r in new if r["n"] == 131072]
    assert len(big) < 0.05 * len(new)
    small = [r["n"] for r in new if r["n"] != 131072]
    assert min(small) >= 64 and max(small) <= 32768
    med = sorted(small)[len(small) // 2]
    assert 700 < med < 2900  # log-uniform on [64, 32768]: median ~ 1448
    by_key = {r["key"]: r for r in new}
    seen = set()
    for r in tr:
        if r["kind"] == 0:
            seen.add(r["key"])
        else:  # a repeat names a matrix already offered, with a fresh right-hand side
            assert r["key"] in seen
            assert r["n"] == by_key[r["key"]]["n"] and r["matrix_seed"] == by_key[r["key"]]["matrix_seed"]
            assert r["rhs_seed"] != by_key[r["key"]]["rhs_seed"]
    assert bench.make_trace(rate, seconds, seed=7) == tr


# ---------------------------------------------------------------- clock record
class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _record(tmp_path, rows):
    p = tmp_path / "clocks.csv"
    p.write_text("".join(", ".join(r) + "\n" for r in rows))
    cs = bench.ClockSampler(0)
    cs.proc, cs.path = _Done(), str(p)
    return cs.stop()


def test_clock_record_power_cap(tmp_path):
    rows = [["0", str(mhz), "2070", "1200.5", "0x4", "Not Active", "Not Active", "Not Active", pc]
            for mhz, pc in ((1950, "Active"), (1980, "Active"), (2010, "Not Active"))]
    c = _record(tmp_path, rows)
    assert c["sm_mhz"] == 1980 and c["sm_max_mhz"] == 2070 and c["samples"] == 3
    assert c["reasons"] == ["sw_power_cap"] and c["power_w_max"] == 1200.5
    assert not os.path.exists(tmp_path / "clocks.csv")


def test_clock_record_thermal(tmp_path):
    rows = [["0", "1500", "2070", "900", "0x40", "Not Active", "Active", "Not Active", "Not Active"],
            ["0", "[N/A]", "2070", "[N/A]", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"]]
    c = _record(tmp_path, rows)
    assert c["reasons"] == ["hw_thermal_slowdown"]
    assert c["sm_mhz"] == 1500 and c["samples"] == 2


def test_clock_record_empty(tmp_path):
    c = _record(tmp_path, [])
    assert c["sm_mhz"] is None and c["reasons"] == ["no samples"]


# ---------------------------------------------------------------- CPU single-request times
def test_cpu_request_times(oracle_mod):
    rows = bench.cpu_request_times(sizes=(64, 200), threads=2)
    assert [r["n"] for r in rows] == [64, 200]
    for r in rows:
        assert r["info"] == 0 and r["seconds"] > 0 and r["nb"] <= r["n"] and r["threads"] == 2
