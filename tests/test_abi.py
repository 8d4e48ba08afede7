"""The C-ABI library: it loads on a host without a GPU, exports every function the
headers declare, keeps the reference's defaults, and reports errors as statuses."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("nomad_gpu.h", "nomad_io.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(nomad_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(ng):
    names = declared_functions()
    assert len(names) >= 20, names
    L = ctypes.CDLL(ng._abi.LIB_PATH)
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    assert names <= set(ng._abi.SIGNATURES), names - set(ng._abi.SIGNATURES)


def test_struct_sizes_match_headers(ng):
    # sizes computed from the header layouts (x86_64 and aarch64 LP64 ABIs agree)
    assert ctypes.sizeof(ng._abi.Params) == 4 + 4 + 8 * 4 + 4 * 14 + 4 * 8
    p = ng.default_params()
    assert p.struct_size == ctypes.sizeof(ng._abi.Params)
    assert ctypes.sizeof(ng._abi.Matrix) == 48
    assert ctypes.sizeof(ng._abi.EpochStats) == 8 * 3 + 4 * 2 + 8 * 5
    assert ctypes.sizeof(ng._abi.CheckpointInfo) == 32
    assert ctypes.sizeof(ng._abi.TuneTrial) == 24


def test_defaults_are_the_references(ng):
    # NomadOption defaults (Code/nomad/nomad_option.cpp:18-47)
    p = ng.default_params()
    assert (p.dim, p.lrate, p.drate, p.reg, p.seed) == (100, 0.001, 0.1, 1.0, 12345)
    assert p.mode == 0 and p.precision == 0 and p.init == 0 and p.init_parts == 1


def test_strerror(ng):
    L = ng.lib()
    assert L.nomad_gpu_strerror(0) == b"ok"
    assert L.nomad_gpu_strerror(-4) == b"device wait timed out"
    assert L.nomad_gpu_strerror(12345) == b"unknown status"


def test_invalid_arguments_are_statuses(ng):
    train, test = ng.synth(ng.synth_spec(1, m=40, n=30, nnz_train=200, nnz_test=20))
    with pytest.raises(ng.NomadError) as e:
        ng.Nomad(train, test, dim=0)
    assert e.value.status == -1
    p = ng.default_params()
    p.struct_size = 12
    with pytest.raises(ng.NomadError) as e:
        ng.Nomad(train, test, params=p)
    assert e.value.status == -1 and "ABI" in str(e.value)


@pytest.mark.parametrize("kw,status,words", [
    (dict(dim=-3), -1, "dim"),
    (dict(init_parts=0), -1, "init_parts"),
    (dict(precision=7), -1, "precision"),
    (dict(lrate=-0.1), -1, "non-negative"),
    (dict(reg=float("nan")), -1, "non-negative"),
    (dict(lr_strategy=5), -1, "lr_strategy"),
    (dict(mode="async", lr_strategy="bold"), -9, "bold driver"),
])
def test_parameters_are_checked_before_any_device_work(ng, kw, status, words):
    """Every parameter check of nomad_gpu_init happens on the host, before the device is
    touched, and names the field; so these run without a GPU."""
    train, test = ng.synth(ng.synth_spec(1, m=40, n=30, nnz_train=200, nnz_test=20))
    with pytest.raises(ng.NomadError) as e:
        ng.Nomad(train, test, **kw)
    assert e.value.status == status
    assert words in str(e.value)


def test_no_device_is_a_status(ng):
    if ng.device_ok(0):
        pytest.skip("a GB300 is present")
    train, test = ng.synth(ng.synth_spec(1, m=40, n=30, nnz_train=200, nnz_test=20))
    with pytest.raises(ng.NomadError) as e:
        ng.Nomad(train, test, dim=8)
    assert e.value.status in (-2, -8)


def test_missing_library_fails_loudly(ng, monkeypatch):
    import nomad_gb300._abi as abi
    monkeypatch.setattr(abi, "_lib", None)
    monkeypatch.setattr(abi, "LIB_PATH", "/nonexistent/libnomad_gpu.so")
    with pytest.raises(ImportError):
        abi.lib()
