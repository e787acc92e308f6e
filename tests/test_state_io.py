"""State files, restart and device snapshots.

The reference writes xms / cps after every step with DelimitedFiles.writedlm
(Analysis.jl:75-78) and restarts from them with readdlm (Input.jl:35-37,
MembraneAleFem.jl:75-107).  These tests pin the library's writer to Julia's
print(::Float64) (known outputs below, and the oracle's restatement of Julia's
shortest printer on seeded doubles of every magnitude), check that readdlm
reads back every double bit for bit and rejects files of the wrong shape, and,
on the GPU, that a run restarted from the files continues bit for bit, that
asynchronous writes capture the state of the step they follow, and that device
snapshots restore exactly.
"""
import math
import os

import numpy as np
import pytest

from _cases import M, O, params_pair, state

# print(::Float64) of Julia (1.10): shortest round-trip digits; fixed notation for
# 1e-4 <= |x| < 1e6, else d.ddd e X
JULIA_PRINT = [
    (1.0, "1.0"), (0.5, "0.5"), (0.1, "0.1"), (0.1 + 0.2, "0.30000000000000004"),
    (1 / 3, "0.3333333333333333"), (2 / 3, "0.6666666666666666"), (12.5, "12.5"),
    (0.0001, "0.0001"), (0.00012, "0.00012"), (1e-5, "1.0e-5"), (1.2e-5, "1.2e-5"),
    (100000.0, "100000.0"), (123456.0, "123456.0"), (12345.678, "12345.678"),
    (1e6, "1.0e6"), (1234567.0, "1.234567e6"), (1e15, "1.0e15"), (-2.5e20, "-2.5e20"),
    (0.0, "0.0"), (-0.0, "-0.0"), (5e-324, "5.0e-324"),
    (1.7976931348623157e308, "1.7976931348623157e308"), (-0.03125, "-0.03125"),
    (math.inf, "Inf"), (-math.inf, "-Inf"), (math.nan, "NaN"),
]


def _seeded_doubles(n, seed=0):
    """Doubles of every binade, plus short decimals and integers."""
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2**63 - 2**52, size=n, dtype=np.int64)  # finite, both signs below
    x = bits.view(np.float64) * np.where(rng.random(n) < 0.5, -1.0, 1.0)
    short = rng.integers(-10**7, 10**7, n) / 10.0 ** rng.integers(0, 8, n)
    ints = rng.integers(-10**7, 10**7, n).astype(np.float64)
    mid = rng.uniform(-2, 2, n) * 10.0 ** rng.integers(-7, 8, n)
    return np.concatenate([x, short, ints, mid])


@pytest.mark.parametrize("x,text", JULIA_PRINT)
def test_oracle_print_matches_julia(x, text):
    assert O.julia_print_float64(x) == text


@pytest.mark.parametrize("x,text", JULIA_PRINT)
def test_format_double_matches_julia(x, text):
    assert M.format_double(x) == text


def test_format_double_matches_oracle_and_round_trips():
    xs = _seeded_doubles(5000)
    for x in xs:
        s = M.format_double(x)
        assert s == O.julia_print_float64(x), (repr(x), s)
        assert float(s.replace("Inf", "inf")) == x


def test_writedlm_text_and_readdlm_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    a = np.asfortranarray(_seeded_doubles(84, seed=4)[:336].reshape(48, 7))
    a[0, 0], a[1, 1], a[2, 2] = 0.0, -0.0, 1e-300
    path = str(tmp_path / "t7-cps.txt")
    M.writedlm(path, a)
    with open(path) as f:
        assert f.read() == O.writedlm_text(a)
    b = M.readdlm(path, 48, 7)
    assert b.tobytes() == a.tobytes()  # bit for bit, signed zero included
    xms = np.asfortranarray(rng.uniform(-1, 1, (5, 3)))
    M.writedlm(path, xms)
    assert M.readdlm(path, 5, 3).tobytes() == xms.tobytes()


def test_readdlm_accepts_readdlm_whitespace(tmp_path):
    path = str(tmp_path / "ws.txt")
    with open(path, "w") as f:
        f.write("1.0 2.5\t\t-3\r\n  4e-3\t5.0e6 6\n\n")
    b = M.readdlm(path, 2, 3)
    assert np.array_equal(b, [[1.0, 2.5, -3.0], [4e-3, 5e6, 6.0]])


def test_readdlm_special_values(tmp_path):
    """What print(::Float64) writes for the special values, a leading '+', and
    numbers beyond the double range (Julia's parse: +-Inf on overflow, +-0 on
    underflow)."""
    path = str(tmp_path / "sp.txt")
    with open(path, "w") as f:
        f.write("+1.5\tInf\t-Inf\nNaN\t1e400\t-1e-400\n-0.0\t5.0e-324\t1.7976931348623157e308\n")
    b = M.readdlm(path, 3, 3)
    assert b[0, 0] == 1.5 and b[0, 1] == np.inf and b[0, 2] == -np.inf
    assert np.isnan(b[1, 0]) and b[1, 1] == np.inf
    assert b[1, 2] == 0.0 and np.signbit(b[1, 2])
    assert b[2, 0] == 0.0 and np.signbit(b[2, 0])
    assert b[2, 1] == 5e-324 and b[2, 2] == np.finfo(np.float64).max


@pytest.mark.parametrize("text,rows,cols", [
    ("1.0\t2.0\n3.0\t4.0\n", 3, 2),   # too few rows
    ("1.0\t2.0\n3.0\t4.0\n", 1, 2),   # too many rows
    ("1.0\t2.0\n3.0\n", 2, 2),        # ragged row
    ("1.0\t2.0\t9\n3.0\t4.0\n", 2, 2),  # too many entries
    ("1.0\tx\n3.0\t4.0\n", 2, 2),     # not a number
    ("1.0\t2.0abc\n3.0\t4.0\n", 2, 2),  # trailing garbage
    ("1.0,2.0\n3.0\t4.0\n", 2, 2),    # not readdlm's separator
    ("+-1.0\t2.0\n3.0\t4.0\n", 2, 2),  # two signs
])
def test_readdlm_rejects_wrong_shape(tmp_path, text, rows, cols):
    path = str(tmp_path / "bad.txt")
    with open(path, "w") as f:
        f.write(text)
    with pytest.raises(M.MafemError):
        M.readdlm(path, rows, cols)


def test_readdlm_missing_file(tmp_path):
    with pytest.raises(M.MafemError):
        M.readdlm(str(tmp_path / "none.txt"), 1, 1)


def test_state_file_names():
    assert M.state_files("out", 12) == (os.path.join("out", "t12-xms.txt"), os.path.join("out", "t12-cps.txt"))
    assert M.f_pull_line([0.5, 1.0, 0.0, 1e-5, -2.0, 0.25, 1e6]) == "0.5\t1.0\t0.0\t1.0e-5\t-2.0\t0.25\t1.0e6"


# ---- GPU ---------------------------------------------------------------------------

DT = 2.0 ** -7  # exact in binary: restarted and uninterrupted runs see the same times


def _setup(motion=M.ALEVB, n=9):
    p, _ = params_pair(motion, M.F_PULL, n, n, pull_speed=0.5)
    mesh = M.Mesh(p)
    xms, cps = state(p, mesh, seed=5, amp=1e-4)
    return p, mesh, xms, cps


@pytest.mark.gpu
@pytest.mark.parametrize("motion", [M.ALEVB, M.LAG])
def test_restart_from_files_continues_bitwise(tmp_path, motion):
    p, mesh, xms, cps = _setup(motion)
    with M.Solver(mesh, p) as a:
        a.upload(xms, cps)
        a.run_analysis([DT] * 4)
        want = a.download()
    d = str(tmp_path)
    with M.Solver(mesh, p) as b:
        b.upload(xms, cps)
        b.run_analysis([DT] * 2)
        b.write_state(d, 2)
        mid = b.download()
    xf, cf = M.state_files(d, 2)
    for f, arr in zip((xf, cf), mid):
        with open(f) as fh:
            assert fh.read() == O.writedlm_text(arr)
    with M.Solver(mesh, p) as c:
        c.read_state(xf, cf)
        got_mid = c.download()
        assert got_mid[0].tobytes() == mid[0].tobytes() and got_mid[1].tobytes() == mid[1].tobytes()
        c.run_analysis([DT] * 2, t0=2 * DT)
        got = c.download()
    assert got[0].tobytes() == want[0].tobytes()
    assert got[1].tobytes() == want[1].tobytes()


@pytest.mark.gpu
def test_async_writes_capture_each_step(tmp_path):
    p, mesh, xms, cps = _setup()
    d = str(tmp_path)
    with M.Solver(mesh, p) as a:
        a.upload(xms, cps)
        a.write_state_async(d, 0)
        for k in range(1, 6):  # no host read of the state between steps
            a.predict(DT)
            a.time_step_resident(k * DT, DT)
            a.write_state_async(d, k)
        a.flush_state_writes()
    with M.Solver(mesh, p) as b:
        b.upload(xms, cps)
        states = [b.download()]
        for k in range(1, 6):
            b.predict(DT)
            b.time_step_resident(k * DT, DT)
            states.append(b.download())
    for k, (x, c) in enumerate(states):
        xf, cf = M.state_files(d, k)
        assert M.readdlm(xf, mesh.numnp, 3).tobytes() == x.tobytes()
        assert M.readdlm(cf, mesh.numnp, mesh.ndf).tobytes() == c.tobytes()
        with open(cf) as fh:
            assert fh.read() == O.writedlm_text(c)


@pytest.mark.gpu
def test_async_write_to_missing_directory_reports_on_flush(tmp_path):
    p, mesh, xms, cps = _setup()
    with M.Solver(mesh, p) as a:
        a.upload(xms, cps)
        a.write_state_async(str(tmp_path / "no" / "such"), 1)
        with pytest.raises(M.MafemError):
            a.flush_state_writes()
        a.flush_state_writes()  # the failure is reported once
        a.write_state(str(tmp_path), 1)
        assert os.path.exists(M.state_files(str(tmp_path), 1)[0])


@pytest.mark.gpu
def test_snapshot_restore_and_retry(tmp_path):
    p, mesh, xms, cps = _setup()
    with M.Solver(mesh, p) as s:
        s.snapshot_reserve(2)
        with pytest.raises(M.MafemError):
            s.snapshot_reserve(3)
        with pytest.raises(M.MafemError):
            s.snapshot(2)
        s.upload(xms, cps)
        s.predict(DT)
        s.time_step_resident(DT, DT)
        s.snapshot(0)
        one = s.download()
        s.predict(DT)
        s.time_step_resident(2 * DT, DT)
        s.snapshot(1)
        two = s.download()
        s.restore(0)
        back = s.download()
        assert back[0].tobytes() == one[0].tobytes() and back[1].tobytes() == one[1].tobytes()
        s.predict(DT)  # retry the second step from the snapshot
        s.time_step_resident(2 * DT, DT)
        again = s.download()
        assert again[0].tobytes() == two[0].tobytes() and again[1].tobytes() == two[1].tobytes()
        s.write_state_async(str(tmp_path), 1, slot=0)
        s.flush_state_writes()
        xf, cf = M.state_files(str(tmp_path), 1)
        assert M.readdlm(cf, mesh.numnp, mesh.ndf).tobytes() == one[1].tobytes()
        assert M.readdlm(xf, mesh.numnp, 3).tobytes() == one[0].tobytes()


@pytest.mark.gpu
def test_pull_record_line():
    p, mesh, xms, cps = _setup()
    with M.Solver(mesh, p) as s:
        s.upload(xms, cps)
        s.run_analysis([DT] * 2)
        rec = s.pull_record(2 * DT)
        x, c = s.download()
        f = s.pull_force()
    # x_pull = sum(xms[IX[:, pull], :], dims=1) / 9 (Analysis.jl:83-84), IX order
    pull = (mesh.numel + 1) // 2 - 1
    nodes = mesh.IX[:, pull] - 1
    want = []
    for j in range(3):
        acc = 0.0
        for nd in nodes:
            acc += x[nd, j]
        want.append(acc / 9)
    assert rec[0] == 2 * DT and rec[1:4] == want and np.array_equal(rec[4:], f)
    assert M.f_pull_line(rec) == "\t".join(O.julia_print_float64(v) for v in rec)
