"""The nomad_gpu driver: the reference's command-line surface (nomad_option.cpp:16-77,
plus --path) and its statistics block (nb_main.cpp:267-285)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "nomad_gb300", "_build", "nomad_gpu")


def run(*args, timeout=300):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=timeout)


def test_help_and_usage(ng):
    r = run("--help")
    assert r.returncode == 1
    for flag in ("--lrate", "--drate", "--reg", "--seed", "--dim", "--timeout", "--input",
                 "--path", "--output", "--nthreads"):
        assert flag in r.stderr


def test_missing_path_is_rejected(ng):
    r = run("--lrate", "0.01")
    assert r.returncode == 1 and "input path has to be specified." in r.stderr


def test_bad_value_and_unknown_option(ng):
    assert run("--path", "x", "--lrate", "abc").returncode == 1
    assert run("--path", "x", "--bogus", "1").returncode == 1
    r = run("--path", "x", "--cptype", "weird")
    assert r.returncode == 1 and "checkpoint type is inalid." in r.stderr


def test_mode_options_are_validated(ng):
    r = run("--path", "x", "--mode", "async", "--lr_strategy", "bold")
    assert r.returncode == 1 and "--lr_strategy bold needs --mode dsgd or dsgdpp." in r.stderr
    assert run("--path", "x", "--mode", "sgd").returncode == 1
    assert "dsgdpp" in run("--help").stderr
    r = run("--path", "x", "--autotune", "many")
    assert r.returncode == 1 and "'--autotune' is invalid" in r.stderr
    assert "--autotune" in run("--help").stderr


def test_checkpoint_options_are_validated(ng):
    """nomad_option.cpp:100-111: a checkpoint type needs a positive interval and a path."""
    r = run("--path", "x", "--cptype", "sync")
    assert r.returncode == 1 and "checkpoint interval is invalid." in r.stderr
    r = run("--path", "x", "--cptype", "SYNC", "-k", "2")
    assert r.returncode == 1 and "checkpoint path is not given." in r.stderr
    for flag in ("--tm_value", "--tm_error", "--tm_interval", "--cpinterval", "--cppath",
                 "--recover"):
        assert flag in run("--help").stderr


def test_unreadable_data_exits_11(ng, tmp_path):
    r = run("--path", str(tmp_path))
    assert r.returncode == 11 and "error in reading training file" in r.stderr


def _write_dataset(ng, d):
    tr, te = ng.synth(ng.synth_spec(1, m=400, n=120, nnz_train=6000, nnz_test=600))
    tr.write(os.path.join(d, "train.dat"))
    te.write(os.path.join(d, "test.dat"))
    return tr, te


@pytest.mark.gpu
def test_end_to_end_run(ng, gpu_ok, tmp_path):
    tr, te = _write_dataset(ng, str(tmp_path))
    out = str(tmp_path / "factors")
    r = run("--path", str(tmp_path), "--dim", "16", "--lrate", "0.01", "--reg", "0.05",
            "--timeout", "0.2", "0.4", "--pause", "0", "--nthreads", "2", "--output", out)
    assert r.returncode == 0, r.stderr
    blocks = re.findall(r"current test RMSE: ([0-9.]+)", r.stdout)
    assert len(blocks) == 2
    m = re.findall(r"detail: train: s=([0-9.]+), c=(\d+); test: s=([0-9.]+), c=(\d+); "
                   r"u=(\d+), f=(\d+), s=(\d+)", r.stdout)
    assert len(m) == 2 and int(m[0][1]) == tr.nnz and int(m[0][3]) == te.nnz
    assert int(m[1][4]) % tr.nnz == 0 and int(m[1][4]) > 0
    lines = open(out + "0").read().splitlines()
    assert len(lines) == tr.m + tr.n
    assert lines[0].startswith("row,0,") and lines[-1].startswith(f"column,{tr.n - 1},")
    assert len(lines[0].split(",")) == 2 + 16


@pytest.mark.gpu
def test_epochs_and_modes(ng, gpu_ok, tmp_path):
    _write_dataset(ng, str(tmp_path))
    for mode in ("async", "replay", "dsgd"):
        r = run("--path", str(tmp_path), "--dim", "8", "--epochs", "2", "--pause", "0",
                "--mode", mode, "--reg", "0.05", "--lrate", "0.01")
        assert r.returncode == 0, (mode, r.stderr)
        rm = float(re.findall(r"current test RMSE: ([0-9.]+)", r.stdout)[0])
        assert np.isfinite(rm)


def _stats(out):
    return re.findall(r"detail: train: s=([0-9.]+), c=(\d+); test: s=([0-9.]+), c=(\d+); "
                      r"u=(\d+), f=(\d+), s=(\d+)", out)


@pytest.mark.gpu
def test_termination_on_small_change(ng, gpu_ok, tmp_path):
    """nb_master.cpp:21-23: the first check always continues (the previous RMSE is
    infinite); a tolerance above any change stops training at the second check, and the
    run ends after one statistics block although more timeout points are listed."""
    tr, _ = _write_dataset(ng, str(tmp_path))
    r = run("--path", str(tmp_path), "--dim", "8", "--lrate", "0.01", "--reg", "0.05",
            "--epochs", "50", "--timeout", "1", "2", "--pause", "0", "--mode", "replay",
            "--tm_interval", "0", "--tm_error", "1e9")
    assert r.returncode == 0, r.stderr
    st = _stats(r.stdout)
    assert len(st) == 1 and int(st[0][4]) == 2 * tr.nnz
    assert r.stderr.count("M: termination check at") == 2
    assert "M: send terimination signal" in r.stderr


@pytest.mark.gpu
def test_termination_on_value_after_eight_passes(ng, gpu_ok, tmp_path):
    """The value condition stops training only once every column made 8 passes."""
    tr, _ = _write_dataset(ng, str(tmp_path))
    r = run("--path", str(tmp_path), "--dim", "8", "--lrate", "0.01", "--reg", "0.05",
            "--epochs", "50", "--pause", "0", "--mode", "replay", "--tm_interval", "0",
            "--tm_error", "0", "--tm_value", "100")
    assert r.returncode == 0, r.stderr
    st = _stats(r.stdout)
    assert len(st) == 1 and int(st[0][4]) == 8 * tr.nnz
    rm = [float(x) for x in re.findall(r"RMSE: ([0-9.]+), difference", r.stderr)]
    assert len(rm) == 8 and all(np.isfinite(rm))


@pytest.mark.gpu
def test_checkpoint_and_recover(ng, gpu_ok, tmp_path):
    """--cptype sync writes cp-t<jobid>-e<k>.ckpt between epochs; --recover k resumes, and
    in replay mode 2 epochs + recover + 1 epoch dumps the same factors as 3 epochs."""
    data, cp = tmp_path / "data", tmp_path / "cp"
    data.mkdir()
    cp.mkdir()
    _write_dataset(ng, str(data))
    common = ("--path", str(data), "--dim", "8", "--lrate", "0.01", "--reg", "0.05",
              "--pause", "0", "--mode", "replay", "--tm_interval", "1e9")
    r = run(*common, "--epochs", "2", "--cptype", "sync", "--cpinterval", "1e-9",
            "--cppath", str(cp), "--jobid", "7")
    assert r.returncode == 0, r.stderr
    assert "Number of checkpoints: 2 " in r.stdout
    assert "Number of archived message in each checkpoint: 0 0" in r.stdout
    assert sorted(os.listdir(cp)) == ["cp-t7-e0.ckpt", "cp-t7-e1.ckpt"]
    assert ng.read_checkpoint(str(cp / "cp-t7-e1.ckpt"))[2] == 2
    r1 = run(*common, "--epochs", "1", "--recover", "1", "--cppath", str(cp), "--jobid", "7",
             "--output", str(tmp_path / "resumed"))
    assert r1.returncode == 0, r1.stderr
    r2 = run(*common, "--epochs", "3", "--output", str(tmp_path / "straight"))
    assert r2.returncode == 0, r2.stderr
    assert open(tmp_path / "resumed0").read() == open(tmp_path / "straight0").read()
    r3 = run(*common, "--epochs", "1", "--recover", "5", "--cppath", str(cp), "--jobid", "7")
    assert r3.returncode == 1 and "error in restoring checkpoint" in r3.stderr


@pytest.mark.gpu
def test_dsgdpp_and_bold_driver_modes(ng, gpu_ok, tmp_path):
    """--mode dsgdpp and --lr_strategy bold (DSGD and DSGD++ only) run end to end."""
    tr, _ = _write_dataset(ng, str(tmp_path))
    for mode, lr in (("dsgdpp", "fixed"), ("dsgdpp", "bold"), ("dsgd", "bold")):
        r = run("--path", str(tmp_path), "--dim", "8", "--epochs", "3", "--pause", "0",
                "--mode", mode, "--lr_strategy", lr, "--reg", "0.05", "--lrate", "0.01")
        assert r.returncode == 0, (mode, lr, r.stderr)
        st = _stats(r.stdout)
        assert int(st[0][4]) == 3 * tr.nnz
    r = run("--path", str(tmp_path), "--mode", "async", "--lr_strategy", "bold")
    assert r.returncode == 1 and "--lr_strategy bold needs --mode dsgd or dsgdpp." in r.stderr


@pytest.mark.gpu
def test_recover_keeps_the_bold_driver_rate(ng, gpu_ok, tmp_path):
    """A DSGD++ bold-driver run resumed from its checkpoint continues with the saved rate
    and objective: its factor dump equals the uninterrupted run's."""
    data, cp = tmp_path / "data", tmp_path / "cp"
    data.mkdir()
    cp.mkdir()
    _write_dataset(ng, str(data))
    common = ("--path", str(data), "--dim", "8", "--lrate", "0.05", "--drate", "0.5", "--reg", "0.05",
              "--pause", "0", "--mode", "dsgdpp", "--lr_strategy", "bold", "--tm_interval", "1e9")
    r = run(*common, "--epochs", "2", "--cptype", "sync", "--cpinterval", "1e-9", "--cppath", str(cp))
    assert r.returncode == 0, r.stderr
    info = ng.read_checkpoint(str(cp / "cp-t1-e1.ckpt"), with_info=True)[2]
    assert info["epochs_done"] == 2 and info["lrate"] > 0 and info["objective"] > 0
    r1 = run(*common, "--epochs", "1", "--recover", "1", "--cppath", str(cp),
             "--output", str(tmp_path / "resumed"))
    assert r1.returncode == 0, r1.stderr
    r2 = run(*common, "--epochs", "3", "--output", str(tmp_path / "straight"))
    assert r2.returncode == 0, r2.stderr
    assert open(tmp_path / "resumed0").read() == open(tmp_path / "straight0").read()


@pytest.mark.gpu
def test_autotune_option(ng, gpu_ok, tmp_path):
    """--autotune N measures the async kernel's configurations (N timed epochs each),
    reports each trial and the choice, then trains with it."""
    _write_dataset(ng, str(tmp_path))
    r = run("--path", str(tmp_path), "--dim", "8", "--epochs", "1", "--pause", "0", "--autotune", "1",
            "--timeout", "1")
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stderr.count("M: autotune trial:") >= 6
    assert "M: autotune: warps per block" in r.stderr
    assert "current test RMSE" in r.stdout
