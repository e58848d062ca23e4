"""Host-side checks of libbna.so that need no GPU: the C ABI exports, the
synthetic generator, the .csr / _ec.nm formats and argument errors."""
import ctypes as C
import hashlib
import json
import os
import re

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
from cuda_newest20160331_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def header_functions():
    src = open(os.path.join(ROOT, "include", "bna.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bna_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_symbol():
    lib = bna.lib()
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes signature table covers the whole header
    assert set(names) == set(L.SIGNATURES)


def test_status_strings():
    lib = bna.lib()
    assert lib.bna_status_string(0) == b"ok"
    assert b"int32" in lib.bna_status_string(3)
    assert lib.bna_version().startswith(b"bna-gb300")


def test_ctx_create_without_gpu_reports_no_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert bna.lib().bna_ctx_create(0, C.byref(h)) == 7  # BNA_NO_DEVICE


def test_synth_is_thread_invariant_and_pinned():
    a = bna.synth_bold(700, 120, 20, 1, threads=1)
    b = bna.synth_bold(700, 120, 20, 1, threads=5)
    assert np.array_equal(a, b)
    assert a.dtype == np.float32 and a.shape == (120, 700)
    # statistics of the factor model: unit noise + 20 * 0.09 loading variance
    assert 2.2 < a.var() < 3.4
    pins = json.load(open(os.path.join(GOLD, "synth_sha256.json")))
    for key, want in pins.items():
        N, T, K, seed, kind = key.split(",")
        x = bna.synth_bold(int(N), int(T), int(K), int(seed), kind=kind,
                           **({"load_sd": 0.117, "jitter_sd": 0.08} if kind == "blocknet" else {}))
        assert hashlib.sha256(x.tobytes()).hexdigest() == want, key


def test_csr_roundtrip_weighted_and_binary(tmp_path):
    rp = np.array([0, 2, 3, 6, 8], np.int32)
    ci = np.array([2, 3, 2, 0, 1, 3, 0, 2], np.int32)
    v = np.linspace(0.1, 0.8, 8).astype(np.float32)
    p = str(tmp_path / "g_weighted.csr")
    bna.csr_write(p, rp, ci, v)
    raw = open(p, "rb").read()
    # int Rlength; R; int Clength; C; int Clength; V  (CorMat.cpp:353-360)
    assert len(raw) == 4 + 5 * 4 + 4 + 8 * 4 + 4 + 8 * 4
    assert np.frombuffer(raw[:4], np.int32)[0] == 5
    r2, c2, v2 = bna.csr_read(p)
    assert np.array_equal(r2, rp) and np.array_equal(c2, ci) and np.array_equal(v2, v)
    pb = str(tmp_path / "g.csr")
    bna.csr_write(pb, rp, ci)
    r3, c3, v3 = bna.csr_read(pb)
    assert v3 is None and np.array_equal(c3, ci)


def test_csr_read_rejects_damaged_files(tmp_path):
    rp = np.array([0, 1, 2], np.int32)
    ci = np.array([1, 0], np.int32)
    v = np.ones(2, np.float32)
    p = str(tmp_path / "a.csr")
    bna.csr_write(p, rp, ci, v)
    raw = bytearray(open(p, "rb").read())
    bad = tmp_path / "bad.csr"
    bad.write_bytes(bytes(raw[:-3]))  # truncated V
    with pytest.raises(bna.BnaError) as e:
        bna.csr_read(str(bad))
    assert e.value.status == 9
    raw2 = bytearray(raw)
    raw2[4 + 12 + 4 + 8: 4 + 12 + 4 + 8 + 4] = np.int32(3).tobytes()  # Vlength != Clength
    bad.write_bytes(bytes(raw2))
    with pytest.raises(bna.BnaError):
        bna.csr_read(str(bad))
    raw3 = bytearray(raw)
    raw3[4 + 12 + 4: 4 + 12 + 8] = np.int32(7).tobytes()  # column out of range
    bad.write_bytes(bytes(raw3))
    with pytest.raises(bna.BnaError):
        bna.csr_read(str(bad))
    with pytest.raises(bna.BnaError) as e:
        bna.csr_read(str(tmp_path / "missing.csr"))
    assert e.value.status == 8


def test_ec_file_format(tmp_path):
    p = str(tmp_path / "x_ec.nm")
    bna.ec_write(p, np.array([1.5, 2.25, -3.0]))
    raw = open(p, "rb").read()
    assert np.frombuffer(raw[:4], np.int32)[0] == 3
    assert np.array_equal(np.frombuffer(raw[4:], np.float32), np.array([1.5, 2.25, -3.0], np.float32))


def test_modu_file_format(tmp_path):
    """_modu.nm (Modularity_CPU.cpp:122-131): int32 N, then the labels as floats."""
    p = str(tmp_path / "x_modu.nm")
    labels = np.array([1, 2, 2, 3, 1], np.int32)
    assert bna.lib().bna_modu_write(p.encode(), labels.ctypes.data, len(labels)) == 0
    raw = open(p, "rb").read()
    assert np.frombuffer(raw[:4], np.int32)[0] == 5
    assert np.array_equal(np.frombuffer(raw[4:], np.float32), labels.astype(np.float32))
    assert bna.lib().bna_modu_write(p.encode(), None, 3) == 1  # BNA_BAD_ARG


def test_bad_arguments_fail_loudly():
    with pytest.raises(ValueError):
        bna._opts("nope", 0.5, "fp32", True, None)
    p = L.SynthParams(N=-1, T=10, K=1)
    assert bna.lib().bna_synth_bold(C.byref(p), None, 1) == 1


def test_request_bytes_estimate_is_monotonic():
    import cuda_newest20160331_gb300 as bna
    small = bna.request_bytes(4096, 240)
    big = bna.request_bytes(45000, 240)
    bigger_t = bna.request_bytes(45000, 1200)
    assert 0 < small < big < bigger_t
    # density mode bounds the CSR by the exact edge count, not the caller's cap
    d = bna.request_bytes(45000, 240, mode="density", value=1.0, cap=10**10)
    assert d < bna.request_bytes(45000, 240, cap=10**10)


def test_server_without_gpu_reports_no_device():
    import ctypes as C
    import torch
    import cuda_newest20160331_gb300 as bna
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert bna.lib().bna_server_create(0, 2, 1 << 30, C.byref(h)) == 7  # BNA_NO_DEVICE


def test_density_nnz_matches_oracle_rule():
    import cuda_newest20160331_gb300 as bna
    import oracle
    for N, s in [(4096, 1.0), (45000, 1.0), (85701, 1.539), (112510, 1.732), (10, 50.0),
                 (180000, 0.1), (3, 0.0)]:
        assert bna.density_nnz(N, s) == 2 * oracle.density_k(N, s), (N, s)


def test_nifti_ingest_gathers_like_the_reference(tmp_path):
    """Mask >= cut in linear voxel order, BOLD[t*N + i] time-major; float and
    double series, uint8 and float masks (CorMat.cpp:141-242)."""
    import numpy as np
    import cuda_newest20160331_gb300 as bna
    from nifti_util import write_nifti
    rng = np.random.default_rng(3)
    Z, Y, X, T = 4, 5, 6, 7
    mask = rng.random((Z, Y, X)).astype(np.float32)
    series = rng.standard_normal((T, Z, Y, X))
    for mdt in (2, 16):
        m = (mask * 2).astype(np.uint8) if mdt == 2 else mask
        write_nifti(tmp_path / "mask.nii", m, mdt)
        cut = 0.5
        sel, N, dims = bna.nifti_mask(str(tmp_path / "mask.nii"), cut)
        flat = m.reshape(-1).astype(np.float32)
        assert dims == (X, Y, Z) and N == int((flat >= np.float32(cut)).sum())
        for ddt in (16, 64):
            write_nifti(tmp_path / "s.nii", series, ddt)
            bold = bna.nifti_bold(str(tmp_path / "s.nii"), sel, N)
            ref = series.reshape(T, -1)[:, flat >= np.float32(cut)].astype(np.float32)
            assert bold.shape == (T, N) and np.array_equal(bold, ref)


def test_nifti_rejects_other_types_and_short_files(tmp_path):
    import numpy as np
    import pytest
    import cuda_newest20160331_gb300 as bna
    from nifti_util import write_nifti
    write_nifti(tmp_path / "m.nii", np.ones((2, 2, 2), np.float64), 64)
    with pytest.raises(bna.BnaError) as e:
        bna.nifti_mask(str(tmp_path / "m.nii"), 0.5)
    assert e.value.status == 9  # BNA_CORRUPT_FILE
    write_nifti(tmp_path / "m.nii", np.ones((2, 2, 2), np.uint8), 2)
    sel, N, _ = bna.nifti_mask(str(tmp_path / "m.nii"), 0.5)
    write_nifti(tmp_path / "s.nii", np.ones((3, 2, 2, 2), np.float32), 16)
    raw = (tmp_path / "s.nii").read_bytes()
    (tmp_path / "s.nii").write_bytes(raw[:-5])
    with pytest.raises(bna.BnaError) as e:
        bna.nifti_bold(str(tmp_path / "s.nii"), sel, N)
    assert e.value.status == 9


def test_cli_usage_and_argument_errors(tmp_path):
    """bna_cormat / bna_cuec print the reference's usage and errors and exit 1
    before touching a device."""
    import os
    import subprocess
    import cuda_newest20160331_gb300 as bna
    b = os.path.join(os.path.dirname(bna.__file__), "bin")
    r = subprocess.run([os.path.join(b, "bna_cormat")], capture_output=True, text=True)
    assert r.returncode == 1 and "Input format" in r.stderr
    r = subprocess.run([os.path.join(b, "bna_cormat"), str(tmp_path), "m.nii", "0.5", "n",
                        "q", "r", "0.3"], capture_output=True, text=True)
    assert r.returncode == 1 and "to_save_cor_matrix type error" in r.stdout
    r = subprocess.run([os.path.join(b, "bna_cormat"), str(tmp_path), "m.nii", "0.5", "n",
                        "n", "x", "0.3"], capture_output=True, text=True)
    assert r.returncode == 1 and "threshold type error" in r.stdout
    r = subprocess.run([os.path.join(b, "bna_cuec")], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([os.path.join(b, "bna_modularity"), str(tmp_path)], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "Input format" in r.stderr
