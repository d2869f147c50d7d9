"""Snapshot files: the reference's dataset names (io/dump_snapshot_impl.hpp,
model/models.cpp, model/all_variables.cpp) in an uncompressed .npz container.

These tests are host-only: the writer and reader need no GPU.  They check the
files against numpy's own .npz reader and writer and Python's zipfile (CRCs),
and the refusals (compressed members, mismatched sizes).
"""
import zipfile

import numpy as np
import pytest

import zisafvm_gb300 as z


def _state(n, na, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, 5)), rng.standard_normal((n, na))


def test_written_file_reads_with_numpy(zlib, tmp_path):
    u, q = _state(37, 2)
    path = tmp_path / "snapshot_0003.npz"
    z.write_snapshot(path, u, t=0.125, n_steps=42, avars=q)
    assert not (tmp_path / "snapshot_0003.npz.tmp").exists()
    with zipfile.ZipFile(path) as zf:
        assert zf.testzip() is None  # every member's CRC-32 matches
        assert all(i.compress_type == zipfile.ZIP_STORED for i in zf.infolist())
    f = np.load(path)
    assert sorted(f.files) == sorted(["time", "n_steps", "rho", "mv1", "mv2", "mv3", "E", "n_avars", "mq0", "mq1"])
    assert f["time"].shape == () and f["time"].dtype == np.float64 and f["time"] == 0.125
    assert f["n_steps"].dtype == np.int64 and f["n_steps"] == 42
    assert f["n_avars"] == 2
    for k, name in enumerate(["rho", "mv1", "mv2", "mv3", "E"]):
        assert f[name].dtype == np.float64 and np.array_equal(f[name], u[:, k])
    for k in range(2):
        assert np.array_equal(f[f"mq{k}"], q[:, k])


def test_numpy_written_file_reads_back(zlib, tmp_path):
    u, q = _state(53, 3, seed=1)
    path = tmp_path / "from_numpy.npz"
    ds = {name: u[:, k] for k, name in enumerate(["rho", "mv1", "mv2", "mv3", "E"])}
    ds.update({f"mq{k}": q[:, k].copy() for k in range(3)})
    np.savez(path, time=np.float64(2.5), n_steps=np.int64(7), n_avars=np.int64(3), **ds)
    r = z.read_snapshot(path)
    assert r["time"] == 2.5 and r["n_steps"] == 7
    assert np.array_equal(r["cvars"], u) and np.array_equal(r["avars"], q)


def test_round_trip_and_steady_state(zlib, tmp_path):
    u, _ = _state(11, 0, seed=2)
    z.write_snapshot(tmp_path / "a.npz", u, t=1.0, n_steps=3)
    r = z.read_snapshot(tmp_path / "a.npz")
    assert np.array_equal(r["cvars"], u) and r["avars"].shape == (11, 0) and (r["time"], r["n_steps"]) == (1.0, 3)
    z.write_snapshot(tmp_path / "steady_state.npz", u)
    assert "time" not in np.load(tmp_path / "steady_state.npz").files
    r = z.read_snapshot(tmp_path / "steady_state.npz")
    assert r["time"] is None and r["n_steps"] is None and np.array_equal(r["cvars"], u)
    # equal states give equal files (fixed member time stamps)
    z.write_snapshot(tmp_path / "b.npz", u, t=1.0, n_steps=3)
    assert (tmp_path / "a.npz").read_bytes() == (tmp_path / "b.npz").read_bytes()


def test_refusals(zlib, tmp_path):
    u, q = _state(9, 1, seed=3)
    ds = {name: u[:, k] for k, name in enumerate(["rho", "mv1", "mv2", "mv3", "E"])}
    np.savez_compressed(tmp_path / "c.npz", time=0.0, n_steps=0, n_avars=0, **ds)
    with pytest.raises(z.ZfvmError, match="compressed"):
        z.read_snapshot(tmp_path / "c.npz")
    (tmp_path / "junk.npz").write_bytes(b"not a zip archive at all, just text")
    with pytest.raises(z.ZfvmError, match="not a zip"):
        z.read_snapshot(tmp_path / "junk.npz")
    with pytest.raises(z.ZfvmError, match="cannot open"):
        z.read_snapshot(tmp_path / "missing.npz")
    z.write_snapshot(tmp_path / "d.npz", u, t=0.0, n_steps=0, avars=q)
    lib = z.load_library()
    out = np.zeros((9, 5))
    # a caller expecting no advected variables is told the file holds one
    assert lib.zfvm_snapshot_read(str(tmp_path / "d.npz").encode(), 9, z._dp(out), 0, None, None, None) != 0
    assert b"advected" in lib.zfvm_last_error()
    assert lib.zfvm_snapshot_read(str(tmp_path / "d.npz").encode(), 8, z._dp(out), 1, z._dp(out), None, None) != 0
    np.savez(tmp_path / "e.npz", time=0.0, n_steps=0, n_avars=0, **{k: v for k, v in ds.items() if k != "E"})
    with pytest.raises(z.ZfvmError, match='"E"'):
        z.read_snapshot(tmp_path / "e.npz")


def test_reader_survives_corrupted_files(zlib, tmp_path):
    """The reader parses files it did not write: truncations, bit flips and
    overwritten header fields must give an error (or, for a flip in the data
    only, a successful read), never a crash."""
    u, q = _state(23, 2, seed=7)
    good = tmp_path / "good.npz"
    z.write_snapshot(good, u, t=1.0, n_steps=2, avars=q)
    data = bytearray(good.read_bytes())
    rng = np.random.default_rng(11)
    bad = tmp_path / "bad.npz"
    trials = 0
    for cut in list(range(0, len(data), max(1, len(data) // 97))) + [len(data) - 1, len(data) - 23]:
        bad.write_bytes(bytes(data[:cut]))
        with pytest.raises(z.ZfvmError):
            z.read_snapshot(bad)
        trials += 1
    for _ in range(400):
        d = bytearray(data)
        for _ in range(int(rng.integers(1, 6))):
            pos = int(rng.integers(0, len(d)))
            d[pos] = int(rng.integers(0, 256)) if rng.random() < 0.5 else d[pos] ^ (1 << int(rng.integers(0, 8)))
        bad.write_bytes(bytes(d))
        try:
            r = z.read_snapshot(bad)
            assert r["cvars"].shape == (23, 5)
        except z.ZfvmError:
            pass
        trials += 1
    # hostile header values: huge sizes, counts and offsets in the zip records
    end = len(data) - 22
    for off, val in ((end + 10, 0xFFFF), (end + 12, 0xFFFFFFFF), (end + 16, 0xFFFFFFFF)):
        d = bytearray(data)
        d[off:off + (2 if val == 0xFFFF else 4)] = val.to_bytes(2 if val == 0xFFFF else 4, "little")
        bad.write_bytes(bytes(d))
        with pytest.raises(z.ZfvmError):
            z.read_snapshot(bad)
        trials += 1
    assert trials > 400
