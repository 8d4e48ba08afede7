"""nomad_gpu_autotune: the measured choice of the ASYNC kernel's runtime configuration
(warps per block, priority threshold, long-visit length) by coordinate descent over fresh
contexts; nomad_gpu_batch_autotune: the batched form's large-problem threshold.  Checked:
the trials they report ran, the configuration returned is the fastest of them, training
with it updates every rating, and what they cannot tune is refused."""
import os
import shutil
import subprocess

import pytest

from test_gpu_parity import LR, DR, REG


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_autotune_picks_the_fastest_trial(ng, gpu_ok, precision):
    train, test = ng.synth(ng.synth_spec(2, m=20000, n=1000, nnz_train=400000, nnz_test=20000, seed=12345))
    kw = dict(dim=32, lrate=LR, drate=DR, reg=REG, mode="async", precision=precision)
    best, trials = ng.autotune(train, test, epochs=1, **kw)
    cap = 10 if precision == "fp32" else 12
    assert len(trials) >= 6
    assert all(t["status"] == 0 and t["device_ms"] > 0 for t in trials)
    assert {t["warps_per_block"] for t in trials} <= {cap, cap - 2, cap - 4}
    assert {t["priority_permille"] for t in trials} >= {25, 50, 100, -1}
    assert {t["long_visit"] for t in trials} >= {10, 14, 20}
    fastest = min(trials, key=lambda t: t["device_ms"])
    chosen = [t for t in trials if (t["warps_per_block"], t["priority_permille"], t["long_visit"]) ==
              (best["warps_per_block"], best["priority_permille"], best["long_visit"])]
    assert chosen and chosen[0]["device_ms"] == fastest["device_ms"]
    with ng.Nomad(train, test, **best) as nm:
        assert nm.epoch(1)["updates"] == train.nnz


def test_autotune_refuses_other_modes(ng):
    """Checked before any device work, so this runs without a GPU."""
    train, test = ng.synth(ng.synth_spec(2, m=2000, n=200, nnz_train=20000, nnz_test=1000, seed=12345))
    for kw in (dict(mode="dsgd"), dict(mode="replay"), dict(mode="async", exact=1)):
        with pytest.raises(ng.NomadError) as e:
            ng.autotune(train, test, dim=16, **kw)
        assert e.value.status == -9
    with pytest.raises(ng.NomadError) as e:
        ng.autotune(train, test, epochs=0, dim=16)
    assert e.value.status == -1


def test_search_on_synthetic_costs(tmp_path):
    """The search itself (nomad_gb300/csrc/tune.h), compiled with g++ against synthetic
    epoch-time models by tests/tune_check.cpp: no GPU."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    exe = str(tmp_path / "tune_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I" + os.path.join(root, "include"),
                    "-I" + os.path.join(root, "nomad_gb300", "csrc"), "-o", exe,
                    os.path.join(here, "tune_check.cpp")], check=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "tune ok" in r.stdout


@pytest.mark.gpu
def test_batch_autotune_picks_the_fastest_share(ng, gpu_ok):
    problems = [ng.synth_batch_problem(i, threads=1) for i in range(96)]
    best, trials = ng.batch_autotune(problems, epochs=2, lrate=0.002, drate=0.1, reg=0.05)
    assert [t["batch_share"] for t in trials] == [1, 2, 4, 8, 16, -1]
    assert all(t["status"] == 0 and t["device_ms"] > 0 for t in trials)
    assert trials[-1]["large_problems"] == 0          # "never": every problem on one warp
    assert (trials[0]["large_problems"] >= trials[1]["large_problems"] >= trials[2]["large_problems"]
            >= trials[3]["large_problems"])
    fastest = min(trials, key=lambda t: t["device_ms"])
    assert best["batch_share"] == fastest["batch_share"]
    nnz = sum(p[0].nnz for p in problems)
    with ng.Batch(problems, **best) as b:
        assert b.epoch(1)["updates"] == nnz


def test_batch_autotune_refusals(ng):
    """Checked before any device work, so this runs without a GPU."""
    problems = [ng.synth_batch_problem(i, threads=1) for i in range(2)]
    with pytest.raises(ng.NomadError) as e:
        ng.batch_autotune(problems, exact=1)
    assert e.value.status == -9
    with pytest.raises(ng.NomadError) as e:
        ng.batch_autotune(problems, epochs=0)
    assert e.value.status == -1
    with pytest.raises(ng.NomadError) as e:
        ng.batch_autotune([])
    assert e.value.status == -1
