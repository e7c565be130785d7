"""Restart files on the host (no GPU): the bundle's framing and index, the
reader's refusals (the reference's load_restart, src/output/restart.cpp
:257-320), and the metadata checks (check_restart_metadata, :322-350)."""
import os

import pytest
import torch

from snapy_gb300 import restart as R


def part(tmp_path, rank, number=3, value=0.0, final=False):
    p = tmp_path / R.part_name("run", rank, number, final)
    R.save_part({"hydro_u": torch.full((5, 1, 4, 8), value + rank,
                                       dtype=torch.float64),
                 "last_time": torch.tensor([1.5]),
                 "last_cycle": torch.tensor([7])}, str(p))
    return p


def test_names():
    assert R.part_name("run", 2, 3) == "run.block2.00003.part"
    assert R.part_name("run", 0, 3, final=True) == "run.block0.final.part"
    assert R.restart_name("run", 12) == "run.00012.restart"
    assert R.part_rank("run.block12.00003.part") == 12
    assert R.part_rank("a.b.block3.final.part") == 3
    assert R.part_rank("run.00003.restart") == -1
    assert R.part_rank("run.blockx.00003.part") == -1


def test_one_part_is_renamed(tmp_path):
    part(tmp_path, 0)
    out = R.combine(str(tmp_path), "run", 3)
    assert os.path.basename(out) == "run.00003.restart"
    assert sorted(os.listdir(tmp_path)) == ["run.00003.restart"]
    d = R.load_restart(out, 0)
    assert torch.equal(d["hydro_u"], torch.zeros(5, 1, 4, 8, dtype=torch.float64))


def test_bundle_round_trip(tmp_path):
    for r in (2, 0, 1):
        part(tmp_path, r, value=10.0)
    out = R.combine(str(tmp_path), "run", 3)
    assert sorted(os.listdir(tmp_path)) == ["run.00003.restart"]  # parts removed
    with open(out, "rb") as f:
        head = f.read(200).split(b"\n")
    assert head[0] == R.BUNDLE_MAGIC.encode() and head[1] == b"3"
    assert [h.split(b"\t")[0] for h in head[2:5]] == [
        b"run.block0.00003.part", b"run.block1.00003.part", b"run.block2.00003.part"]
    assert head[5] == b""
    for r in range(3):
        d = R.load_restart(out, r)
        assert float(d["hydro_u"][0, 0, 0, 0]) == 10.0 + r
        assert int(d["last_cycle"]) == 7


def bundle_bytes(tmp_path):
    for r in (0, 1):
        part(tmp_path, r)
    return open(R.combine(str(tmp_path), "run", 3), "rb").read()


@pytest.mark.parametrize("mutate, message", [
    (lambda b: b.replace(b"\n2\n", b"\n\n", 1), "missing entry count"),
    (lambda b: b.replace(b".part\t", b".part ", 1), "missing tab"),
    (lambda b: b.replace(b"\n\n", b"\nx\n", 1), "missing terminator"),
    (lambda b: b[:-100], "truncated"),
])
def test_malformed_bundles_are_refused(tmp_path, mutate, message):
    data = mutate(bundle_bytes(tmp_path))
    bad = tmp_path / "bad.restart"
    bad.write_bytes(data)
    rank = 1 if message == "truncated" else 0
    with pytest.raises(R.RestartError, match=message):
        R.load_restart(str(bad), rank)


def test_missing_block_and_file(tmp_path):
    data = bundle_bytes(tmp_path)
    f = tmp_path / "ok.restart"
    f.write_bytes(data)
    with pytest.raises(R.RestartError, match="no part for block 5"):
        R.load_restart(str(f), 5)
    with pytest.raises(R.RestartError, match="failed to open"):
        R.load_restart(str(tmp_path / "absent.restart"))


def meta_data(bits=32):
    dt = torch.float32 if bits == 32 else torch.float64
    grid = [torch.linspace(0, 1, 9, dtype=torch.float64),
            torch.linspace(0, 2, 5, dtype=torch.float64),
            torch.linspace(0, 1, 2, dtype=torch.float64)]
    d = {"hydro_u": torch.zeros(5, 1, 4, 8, dtype=torch.float64),
         "hydro_u_stored": torch.zeros(5, 1, 4, 8, dtype=dt),
         "hydro_ref": torch.zeros(41, dtype=torch.float64),
         R.HYDRO_RESTART_METADATA: torch.tensor([1, bits], dtype=torch.int64)}
    for k, g in zip(R.HYDRO_REFERENCE_GRID, grid):
        d[k] = g.clone()
    return d, grid


def test_metadata_checks():
    d, grid = meta_data()
    R.check_restart_metadata(d, grid)
    bad = dict(d)
    bad[R.HYDRO_RESTART_METADATA] = torch.tensor([2, 32], dtype=torch.int64)
    with pytest.raises(R.RestartError, match="version"):
        R.check_restart_metadata(bad, grid)
    bad = dict(d)
    bad[R.HYDRO_RESTART_METADATA] = torch.tensor([1, 64], dtype=torch.int64)
    with pytest.raises(R.RestartError, match="dtype/shape"):
        R.check_restart_metadata(bad, grid)
    bad = dict(d)
    del bad["hydro_ref"]
    with pytest.raises(R.RestartError, match="requires hydro_ref"):
        R.check_restart_metadata(bad, grid)
    moved = [grid[0] + 1e-12, grid[1], grid[2]]
    with pytest.raises(R.RestartError, match="reference grid mismatch at hydro_ref_x1f"):
        R.check_restart_metadata(d, moved)
    with pytest.raises(R.RestartError, match="perturbation-flux"):
        R.check_restart_metadata(d, grid, perturbation_flux=True)


def test_required_variables():
    with pytest.raises(R.RestartError, match="missing required variable: next_time"):
        R.require({"hydro_u": 0, "last_time": 0, "last_cycle": 0, "file_number": 0})


def test_budget_carry_keys_round_trip():
    """write_budget_carry / read_budget_carry (src/output/restart.cpp
    :383-407): the six budget_carry.* keys, the row names packed as one
    newline-terminated int8 tensor; a carry with other rows, or a file
    without one, starts a new interval (None)."""
    import numpy as np
    from snapy_gb300 import budget as Bg
    c = Bg.BudgetCarry(rows=list(Bg.ROWS), total_prev=np.arange(5.0),
                       pending=np.full(5, 0.5),
                       counter=np.arange(len(Bg.COUNTERS), dtype=np.int64),
                       minimum=np.full(len(Bg.MINIMA), np.inf), interval=1.25)
    out = {}
    Bg.write_budget_carry(c, out)
    assert sorted(out) == sorted(Bg.CARRY_PREFIX + k for k in (
        "rows", "total_prev", "pending", "counter", "minimum", "interval"))
    assert out[Bg.CARRY_PREFIX + "rows"].dtype == torch.int8
    assert bytes(out[Bg.CARRY_PREFIX + "rows"].view(torch.uint8).tolist()) == \
        ("\n".join(Bg.ROWS) + "\n").encode()
    back = Bg.read_budget_carry(out, Bg.ROWS)
    assert back.rows == Bg.ROWS and back.interval == 1.25
    assert np.array_equal(back.total_prev, c.total_prev)
    assert np.array_equal(back.counter, c.counter)
    assert np.isinf(back.minimum).all()
    assert Bg.read_budget_carry(out, Bg.ROWS[:4]) is None
    del out[Bg.CARRY_PREFIX + "pending"]
    assert Bg.read_budget_carry(out, Bg.ROWS) is None
    Bg.write_budget_carry(None, out)  # an undefined carry writes nothing
