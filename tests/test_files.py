"""Raw binary files of the host side (include/lgame_host.h): restart snapshots and lateral
boundary levels, where the reference uses netCDF.

CPU: round trips, the documented little-endian header, rejection of files of the wrong kind,
dimensions or length, read_boundaries' file names, a run resumed from a snapshot file that
continues bit for bit (oracle), and boundary levels read from files instead of memory.  GPU:
the same resume in both precisions, and the library's own file loader in the step.
"""
import struct

import numpy as np
import pytest

import cases
import lgame_gpu as L
import oracle as O
from test_boundaries import _level, _namelist


def _dims(hm):
    return hm.ny, hm.nx, hm.nl, hm.ncons


def _oracle_run(key, nsteps, cfg=None):
    n = _namelist(key)
    hm = L.HostModel(n)
    o = O.Oracle(cfg or L.config_from_namelist(n), hm.grid)
    o.set_state(0, hm.state)
    o.set_state(1, hm.state)
    o.set_diag(hm.diag)
    for k in range(nsteps):
        o.pchevi(k % 2, (k + 1) % 2, k)
    return hm, o


def test_snapshot_round_trip_and_header(tmp_path):
    hm, o = _oracle_run("jet", 2)
    s0, s1, dg = o.get_state(0), o.get_state(1), o.get_diag()
    path = tmp_path / "run.snap"
    L.write_snapshot(path, *_dims(hm), 2, s0, s1, dg, ns=hm.ns)
    step, r0, r1, rd = L.read_snapshot(path, *_dims(hm), ns=hm.ns)
    assert step == 2
    for a, b in ((s0, r0), (s1, r1), (dg, rd)):
        for f in a:
            np.testing.assert_array_equal(a[f], b[f], err_msg=f)
    raw = path.read_bytes()
    magic, version, ny, nx, nl, nc, st, ns = struct.unpack_from("<8s5iqi", raw, 0)
    assert (magic, version, ny, nx, nl, nc, st, ns) == (b"LGAMESNP", 4, hm.ny, hm.nx, hm.nl, hm.ncons, 2, hm.ns)
    assert raw[40:64] == bytes(24)
    n_doubles = 2 * sum(v.size for v in s0.values()) + sum(v.size for v in dg.values())
    assert len(raw) == 64 + 8 * n_doubles
    first = np.frombuffer(raw, dtype="<f8", count=4, offset=64)
    np.testing.assert_array_equal(first, s0["rho"].ravel(order="F")[:4])
    o.close()


def test_files_reject_wrong_kind_dims_and_length(tmp_path):
    hm, o = _oracle_run("hills_nonperiodic", 0)
    d = _dims(hm)
    s, dg = o.get_state(0), o.get_diag()
    snap = tmp_path / "a.snap"
    L.write_snapshot(snap, *d, 0, s, s, dg, ns=hm.ns)
    with pytest.raises(L.LgameError) as e:
        L.read_snapshot(snap, d[0] + 1, d[1], d[2], d[3], ns=hm.ns)
    assert e.value.code == L.ERR_BAD_DIMS
    with pytest.raises(L.LgameError) as e:      # other number of soil layers
        L.read_snapshot(snap, *d, ns=hm.ns + 1)
    assert e.value.code == L.ERR_BAD_DIMS
    lev = tmp_path / "bc+0s.bin"
    L.write_bc_level(lev, *d, 0.0, _level(hm, 0.0))
    with pytest.raises(L.LgameError):
        L.read_snapshot(lev, *d, ns=hm.ns)    # a boundary level is not a snapshot
    with pytest.raises(L.LgameError):
        L.read_bc_level(snap, *d)             # and the other way round
    raw = snap.read_bytes()
    (tmp_path / "short.snap").write_bytes(raw[:-8])
    (tmp_path / "long.snap").write_bytes(raw + b"\0")
    for name in ("short.snap", "long.snap"):
        with pytest.raises(L.LgameError):
            L.read_snapshot(tmp_path / name, *d, ns=hm.ns)
    with pytest.raises(L.LgameError):
        L.read_snapshot(tmp_path / "missing.snap", *d, ns=hm.ns)
    o.close()


def test_bc_level_round_trip_and_names(tmp_path):
    hm, o = _oracle_run("hills_nonperiodic", 0)
    lev = _level(hm, 30.0)
    L.write_bc_level(tmp_path / "x.bin", *_dims(hm), 30.0, lev)
    t, r = L.read_bc_level(tmp_path / "x.bin", *_dims(hm))
    assert t == 30.0
    for f in L.BC_FIELDS:
        np.testing.assert_array_equal(r[f], lev[f], err_msg=f)
    # int(t_update - t_init), truncated toward zero, as read_boundaries forms it
    assert L.bc_filename("bc", 1577836800.0 + 10800.0, 1577836800.0) == "bc+10800s.bin"
    assert L.bc_filename("dir/bc", 15.9, 0.0) == "dir/bc+15s.bin"
    assert L.bc_filename("bc", -0.5, 0.0) == "bc+0s.bin"
    o.close()


@pytest.mark.parametrize("key", ["jet", "hills_nonperiodic"])
def test_oracle_resume_from_snapshot_is_bit_identical(key, tmp_path):
    """Four steps in one go against two steps, a snapshot file, a fresh context and two more.
    The non-periodic case keeps edge values of the state it overwrites, so both slots matter."""
    hm, ref = _oracle_run(key, 4)
    hm2, o = _oracle_run(key, 2)
    L.write_snapshot(tmp_path / "s.snap", *_dims(hm2), 2, o.get_state(0), o.get_state(1), o.get_diag(), ns=hm2.ns)
    o.close()
    step, s0, s1, dg = L.read_snapshot(tmp_path / "s.snap", *_dims(hm2), ns=hm2.ns)
    r = O.Oracle(L.config_from_namelist(_namelist(key)), hm2.grid)
    r.set_state(0, s0)
    r.set_state(1, s1)
    r.set_diag(dg)
    for k in range(step, 4):
        r.pchevi(k % 2, (k + 1) % 2, k)
    for slot in (0, 1):
        a, b = ref.get_state(slot), r.get_state(slot)
        for f in L.STATE_FIELDS:
            np.testing.assert_array_equal(a[f], b[f], err_msg=f"{key} slot {slot} {f}")
    da, db = ref.get_diag(), r.get_diag()
    for f in L.DIAG_FIELDS:
        np.testing.assert_array_equal(da[f], db[f], err_msg=f)
    ref.close()
    r.close()


def test_oracle_boundary_levels_from_files(tmp_path):
    """The relaxation with its levels read from files equals the one fed from memory."""
    n = _namelist("hills_nonperiodic")
    hm = L.HostModel(n)
    d = _dims(hm)
    for t in (0.0, 15.0, 30.0, 45.0, 60.0):
        L.write_bc_level(tmp_path / L.bc_filename("bc", t, 0.0), *d, t, _level(hm, t))
    root = str(tmp_path / "bc")
    out = []
    for from_files in (True, False):
        o = O.Oracle(L.config_from_namelist(n), hm.grid)
        o.set_state(0, hm.state)
        o.set_state(1, hm.state)
        o.set_diag(hm.diag)
        if from_files:
            o.bc_setup(3, 15, 0.0, lambda t, idx: L.read_bc_level(L.bc_filename(root, t, 0.0), *d)[1])
            o.set_bc(1, L.read_bc_level(L.bc_filename(root, 0.0, 0.0), *d)[1])
            o.set_bc(2, L.read_bc_level(L.bc_filename(root, 15.0, 0.0), *d)[1])
        else:
            o.bc_setup(3, 15, 0.0, lambda t, idx: _level(hm, t))
            o.set_bc(1, _level(hm, 0.0))
            o.set_bc(2, _level(hm, 15.0))
        for k in range(5):
            o.pchevi(k % 2, (k + 1) % 2, k)
        out.append((o.get_state(1), o.bc_state()))
        o.close()
    assert out[0][1] == out[1][1]
    for f in L.STATE_FIELDS:
        np.testing.assert_array_equal(out[0][0][f], out[1][0][f], err_msg=f)


# ---- GPU ------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("precision", [L.PRECISION_FP64, L.PRECISION_SPLIT])
def test_gpu_resume_from_snapshot_is_bit_identical(precision, tmp_path):
    n = _namelist("jet")
    hm = L.HostModel(n)
    cfg = L.config_from_namelist(n)
    cfg.precision = precision

    def fresh():
        g = L.GpuModel(cfg, hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        return g
    ref = fresh()
    for k in range(4):
        ref.pchevi(k % 2, (k + 1) % 2, k)
    g = fresh()
    for k in range(2):
        g.pchevi(k % 2, (k + 1) % 2, k)
    L.write_snapshot(tmp_path / "s.snap", *_dims(hm), 2, g.get_state(0), g.get_state(1), g.get_diag(), ns=hm.ns)
    g.close()
    step, s0, s1, dg = L.read_snapshot(tmp_path / "s.snap", *_dims(hm), ns=hm.ns)
    r = L.GpuModel(cfg, hm.grid)
    r.set_state(0, s0)
    r.set_state(1, s1)
    r.set_diag(dg)
    for k in range(step, 4):
        r.pchevi(k % 2, (k + 1) % 2, k)
    for slot in (0, 1):
        a, b = ref.get_state(slot), r.get_state(slot)
        for f in L.STATE_FIELDS:
            np.testing.assert_array_equal(a[f], b[f], err_msg=f"slot {slot} {f}")
    ref.close()
    r.close()


@pytest.mark.gpu
def test_gpu_boundary_levels_from_files(tmp_path):
    """lgame_bc_file_loader in the step against levels handed over from memory."""
    n = _namelist("hills_nonperiodic")
    hm = L.HostModel(n)
    d = _dims(hm)
    for t in (0.0, 15.0, 30.0, 45.0, 60.0):
        L.write_bc_level(tmp_path / L.bc_filename("bc", t, 0.0), *d, t, _level(hm, t))
    root = str(tmp_path / "bc")
    out = []
    for from_files in (True, False):
        g = L.GpuModel(L.config_from_namelist(n), hm.grid)
        g.set_state(0, hm.state)
        g.set_state(1, hm.state)
        g.set_diag(hm.diag)
        if from_files:
            g.bc_setup_files(3, 15, root, 0.0)
        else:
            g.bc_setup(3, 15, 0.0, lambda t, idx: _level(hm, t))
        g.set_bc(1, _level(hm, 0.0))
        g.set_bc(2, _level(hm, 15.0))
        for k in range(5):
            g.pchevi(k % 2, (k + 1) % 2, k)
        out.append((g.get_state(1), g.bc_state()))
        g.close()
    assert out[0][1] == out[1][1] and out[0][1][2] > 0.0
    for f in L.STATE_FIELDS:
        np.testing.assert_array_equal(out[0][0][f], out[1][0][f], err_msg=f)
