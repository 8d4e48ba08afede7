"""Checkpoint / resume at epoch boundaries.

The reference archives each worker thread's rows (NomadBody::archive_local,
nb_checkpoint.cpp:47-59) plus the column messages queued at the cut
(nb_checkpoint.cpp:61-102) and restores them with --recover (nb_main.cpp:446-449).
Between epochs no column token is in flight, so the factors and the pass count are
the whole state; a context restored from the checkpoint of epoch k and trained on
continues exactly as one that never stopped:
  * file format (CPU): layout, FNV-1a 64 hash, atomic replace, every error status;
  * REPLAY and DSGD (GPU): k epochs + checkpoint + restore + e epochs equals k + e
    epochs bit for bit, fp32 and bf16;
  * ASYNC (GPU): the pass count carries over; RMSE matches the uninterrupted run.
"""
import os
import struct

import numpy as np
import pytest

LR, DR, REG = 0.01, 0.1, 0.05


def fnv1a64(data):
    h = 14695981039346656037
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def rand_factors(m, n, dim, seed=1):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((m, dim)).astype(np.float32),
            rng.standard_normal((n, dim)).astype(np.float32))


def test_round_trip_and_layout(ng, tmp_path):
    W, H = rand_factors(7, 5, 3)
    p = str(tmp_path / "cp.ckpt")
    ng.write_checkpoint(p, W, H, 4, lrate=0.0125, objective=321.5)
    W2, H2, info = ng.read_checkpoint(p, with_info=True)
    assert info == dict(m=7, n=5, dim=3, epochs_done=4, lrate=0.0125, objective=321.5)
    assert np.array_equal(W, W2) and np.array_equal(H, H2)
    raw = open(p, "rb").read()
    assert raw[:8] == b"NOMADCP1"
    assert struct.unpack("<iiiidd", raw[8:40]) == (7, 5, 3, 4, 0.0125, 321.5)
    payload = W.tobytes() + H.tobytes()
    assert struct.unpack("<Q", raw[40:48])[0] == fnv1a64(raw[8:40] + payload)
    assert raw[48:] == payload
    ng.write_checkpoint(p, W, H, 1)  # no bold-driver state
    assert ng.read_checkpoint(p, with_info=True)[2]["objective"] == -1.0
    assert not os.path.exists(p + ".tmp")


def test_replace_and_empty_sides(ng, tmp_path):
    p = str(tmp_path / "cp.ckpt")
    W, H = rand_factors(4, 0, 2)
    ng.write_checkpoint(p, W, H, 0)
    W2, H2, ep = ng.read_checkpoint(p)
    assert W2.shape == (4, 2) and H2.shape == (0, 2) and ep == 0 and np.array_equal(W, W2)
    W, H = rand_factors(3, 6, 2, seed=2)
    ng.write_checkpoint(p, W, H, 9)  # replaces the file in place
    W2, H2, ep = ng.read_checkpoint(p)
    assert ep == 9 and np.array_equal(H, H2)


def test_format_errors(ng, tmp_path):
    W, H = rand_factors(6, 4, 3)
    good = tmp_path / "good.ckpt"
    ng.write_checkpoint(str(good), W, H, 2)
    raw = good.read_bytes()

    def status(data=None, path=None, **kw):
        if path is None:
            path = tmp_path / "x.ckpt"
            path.write_bytes(data)
        with pytest.raises(ng.NomadError) as e:
            if kw:
                Wb = np.empty((kw["m"], kw["dim"]), np.float32)
                Hb = np.empty((kw["n"], kw["dim"]), np.float32)
                ng.check(ng.lib().nomad_io_read_checkpoint(os.fsencode(str(path)), kw["m"], kw["n"],
                                                           kw["dim"], Wb.ctypes.data, Hb.ctypes.data,
                                                           None), "read")
            else:
                ng.read_checkpoint(str(path))
        return e.value.status

    assert status(b"NOMADCPX" + raw[8:]) == -7                      # magic
    assert status(raw[:44]) == -7                                   # short header
    assert status(raw[:-4]) == -7                                   # short payload
    assert status(raw + b"\0") == -7                                # trailing bytes
    for pos in (30, 60):                                            # hash: header, payload
        flip = bytearray(raw)
        flip[pos] ^= 1
        assert status(bytes(flip)) == -7
    neg = bytearray(raw)
    neg[8:12] = struct.pack("<i", -1)
    assert status(bytes(neg)) == -7                                 # negative size
    assert status(path=tmp_path / "missing.ckpt") == -6             # no file
    assert status(path=good, m=5, n=4, dim=3) == -1                 # other problem
    assert status(path=good, m=6, n=4, dim=2) == -1


def test_write_rejects_bad_arguments(ng, tmp_path):
    W, H = rand_factors(2, 2, 2)
    with pytest.raises(ng.NomadError) as e:
        ng.write_checkpoint(str(tmp_path / "a"), W, H, -1)
    assert e.value.status == -1
    with pytest.raises(ng.NomadError) as e:
        ng.write_checkpoint(str(tmp_path / "no_such_dir" / "a"), W, H, 0)
    assert e.value.status == -6


def _problem(ng, seed=3):
    spec = ng.synth_spec(1, m=900, n=260, nnz_train=30000, nnz_test=3000)
    spec.seed = seed
    return ng.synth(spec)


@pytest.mark.gpu
@pytest.mark.parametrize("mode,precision", [("replay", "fp32"), ("replay", "bf16"),
                                            ("dsgd", "fp32"), ("dsgd", "bf16")])
def test_resume_is_bit_exact(ng, gpu_ok, tmp_path, mode, precision):
    train, test = _problem(ng)
    kw = dict(dim=16, lrate=LR, drate=DR, reg=REG, mode=mode, precision=precision)
    with ng.Nomad(train, test, **kw) as a:
        a.epoch(3)
        Wa, Ha = a.factors()
    p = str(tmp_path / "cp.ckpt")
    with ng.Nomad(train, test, **kw) as b:
        b.epoch(2)
        b.save_checkpoint(p)
    assert ng.read_checkpoint(p)[2] == 2
    with ng.Nomad(train, test, **kw) as c:
        c.load_checkpoint(p)
        st = c.epoch(1)
        Wc, Hc = c.factors()
    assert st["epochs_done"] == 3 and np.isfinite(Wa).all()
    assert np.array_equal(Wa, Wc) and np.array_equal(Ha, Hc)


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [0, 1])
def test_async_resume_carries_pass_count(ng, gpu_ok, tmp_path, exact):
    train, test = _problem(ng, seed=4)
    kw = dict(dim=32, lrate=LR, drate=DR, reg=REG, mode="async", exact=exact)
    with ng.Nomad(train, test, **kw) as a:
        a.epoch(4)
        ra = a.rmse()[1]
    p = str(tmp_path / "cp.ckpt")
    with ng.Nomad(train, test, **kw) as b:
        b.epoch(2)
        b.save_checkpoint(p)
        Wb, Hb = b.factors()
    with ng.Nomad(train, test, **kw) as c:
        c.load_checkpoint(p)
        W0, H0 = c.factors()
        assert np.array_equal(W0, Wb) and np.array_equal(H0, Hb)
        st = c.epoch(2)
        rc = c.rmse()[1]
    assert st["epochs_done"] == 4 and st["updates"] == 2 * train.nnz
    assert abs(rc - ra) <= 0.005 * ra, (rc, ra)


@pytest.mark.gpu
def test_set_epochs_done_sets_the_step(ng, gpu_ok):
    """Epoch k+1 from given factors equals the same epoch of an uninterrupted run once
    the pass count is set; with the count left at 0 it does not (larger step)."""
    train, test = _problem(ng, seed=5)
    kw = dict(dim=8, lrate=LR, drate=DR, reg=REG, mode="replay")
    with ng.Nomad(train, test, **kw) as a:
        a.epoch(2)
        W2, H2 = a.factors()
        a.epoch(1)
        W3, H3 = a.factors()
    with ng.Nomad(train, test, W0=W2, H0=H2, **kw) as b:
        b.set_epochs_done(2)
        b.epoch(1)
        assert np.array_equal(b.factors()[0], W3)
    with ng.Nomad(train, test, W0=W2, H0=H2, **kw) as c:
        c.epoch(1)
        assert not np.array_equal(c.factors()[0], W3)


@pytest.mark.gpu
def test_load_rejects_mismatched_checkpoints(ng, gpu_ok, tmp_path):
    """A checkpoint of another shape, or one without bold-driver state for a bold-driver
    context, is an invalid argument and leaves the context usable."""
    train, test = _problem(ng, seed=6)
    p = str(tmp_path / "cp.ckpt")
    with ng.Nomad(train, test, dim=8, lrate=LR, drate=DR, reg=REG, mode="replay") as a:
        a.epoch(1)
        a.save_checkpoint(p)
    with ng.Nomad(train, test, dim=16, lrate=LR, drate=DR, reg=REG, mode="replay") as b:
        with pytest.raises(ng.NomadError) as e:
            b.load_checkpoint(p)
        assert e.value.status == -1
        assert b.epoch(1)["epochs_done"] == 1
    with ng.Nomad(train, test, dim=8, lrate=LR, drate=0.5, reg=REG, mode="dsgd",
                  lr_strategy="bold", dsgd_inner_blocks=4) as c:
        with pytest.raises(ng.NomadError) as e:
            c.load_checkpoint(p)
        assert e.value.status == -1 and "bold-driver" in str(e.value)
        assert c.epoch(1)["epochs_done"] == 1
