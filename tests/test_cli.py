"""Command-line drop-ins: bna_cormat (CUCorMat's arguments and outputs,
W/CorMat/CUCorMat/CUCorMat/CorMat.cpp:52-670), bna_cormat_u (the unweighted
tree's CUCorMat, U/CorMat/CUCorMat/CUCORMAT/CorMat.cpp) and bna_cuec (CUEC,
W/CUEC/weighted-net.cu:222-331), run on NIfTI files written here; outputs
checked against the oracle."""
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import cuda_newest20160331_gb300 as bna
import oracle
from nifti_util import write_nifti

pytestmark = pytest.mark.gpu
BIN = os.path.join(os.path.dirname(bna.__file__), "bin")


def _subjects(tmp_path):
    rng = np.random.default_rng(5)
    Z, Y, X = 8, 10, 12
    mask = (rng.random((Z, Y, X)) < 0.6).astype(np.uint8)
    N = int(mask.sum())
    sel = mask.reshape(-1).astype(bool)
    bolds = []
    for k, (T, dt) in enumerate([(80, 16), (100, 64)]):
        b = bna.synth_bold(N, T, 10, 300 + k)
        vol = np.zeros((T, Z * Y * X), np.float64 if dt == 64 else np.float32)
        vol[:, sel] = b
        write_nifti(tmp_path / f"s{k + 1}.nii", vol.reshape(T, Z, Y, X), dt)
        bolds.append(b)
    write_nifti(tmp_path / "mask.nii", mask, 2)
    return N, bolds


def _run(*args):
    r = subprocess.run([os.path.join(BIN, args[0]), *map(str, args[1:])], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_cormat_and_cuec_end_to_end(tmp_path):
    N, bolds = _subjects(tmp_path)
    M1 = N * (N - 1) // 2
    _run("bna_cormat", tmp_path, tmp_path / "mask.nii", 0.5, "bn", "y", "r", 0.3, 0.4)
    for k, b in enumerate(bolds, 1):
        for tau in (0.3, 0.4):
            R, C, V = oracle.csr_corr(b, "r_gt", tau)
            spa = 100.0 * len(C) / M1 / 2
            f = tmp_path / "weighted" / f"s{k}_{N}_spa{spa:.3f}%_cor{tau:.3f}_weighted.csr"
            assert f.exists(), sorted(os.listdir(tmp_path / "weighted"))
            rp, ci, va = bna.csr_read(str(f))
            assert np.array_equal(rp, R) and np.array_equal(ci, C)
        cm = np.fromfile(tmp_path / "weighted" / f"s{k}_{N}.cormat", np.float32, offset=4)
        ref = oracle.cormat_packed(oracle.zscore(b))
        assert len(cm) == M1 and np.max(np.abs(cm - ref)) < 1e-3
    # the average (second letter n: plain)
    A = oracle.avg_packed(bolds)
    for tau in (0.3, 0.4):
        R, C, V = oracle.threshold_csr(A, N, "r_gt", tau)
        spa = 100.0 * len(C) / M1 / 2
        f = tmp_path / f"{tmp_path.name}_2_{N}_spa{spa:.3f}%_cor{tau:.3f}.csr"
        assert f.exists(), sorted(os.listdir(tmp_path))
        rp, ci, va = bna.csr_read(str(f))
        assert np.array_equal(rp, R) and np.array_equal(ci, C)
    # centrality of every written .csr
    _run("bna_cuec", tmp_path / "weighted")
    for f in glob.glob(str(tmp_path / "weighted" / "*.csr")):
        rp, ci, va = bna.csr_read(f)
        e, lam, it, conv = oracle.ec(rp, ci, va.astype(np.float64))
        stem = f[:-4]
        raw = np.fromfile(stem + "_ec.nm", np.int32, count=1)
        ec = np.fromfile(stem + "_ec.nm", np.float32, offset=4)
        assert raw[0] == N and len(ec) == N
        assert np.max(np.abs(ec - e)) <= 1e-5 * np.max(np.abs(e)) + 1e-6
        lam_txt = float(open(stem + "_evalue.txt").read())
        assert abs(lam_txt - lam) <= 1e-5 * abs(lam)


def test_cormat_density_mode(tmp_path):
    N, bolds = _subjects(tmp_path)
    out = _run("bna_cormat", tmp_path, tmp_path / "mask.nii", 0.5, "n", "n", "s", 2.5)
    z = oracle.zscore(bolds[0])
    tau, k, drop = oracle.density(oracle.cormat_packed(z), N, 2.5)
    f = glob.glob(str(tmp_path / "weighted" / f"s1_{N}_spa2.500%_cor*_weighted.csr"))
    assert len(f) == 1, out
    assert re.search(rf"_cor{np.float32(tau):.3f}_weighted", f[0])
    rp, ci, va = bna.csr_read(f[0])
    assert len(ci) == 2 * k


def test_unweighted_tree_cormat(tmp_path):
    """bna_cormat_u (U/CorMat/CUCorMat/CUCORMAT/CorMat.cpp): the same
    arguments, per-subject files in Dir/unweighted without the _weighted
    suffix, binary .csr (no value section); r and density thresholds; the
    binary files feed bna_cuec like the reference's unweighted CUEC."""
    N, bolds = _subjects(tmp_path)
    M1 = N * (N - 1) // 2
    _run("bna_cormat_u", tmp_path, tmp_path / "mask.nii", 0.5, "n", "n", "r", 0.3, 0.45)
    for k, b in enumerate(bolds, 1):
        for tau in (0.3, 0.45):
            R, C, _ = oracle.csr_corr(b, "r_gt", tau)
            spa = 100.0 * len(C) / M1 / 2
            f = tmp_path / "unweighted" / f"s{k}_{N}_spa{spa:.3f}%_cor{tau:.3f}.csr"
            assert f.exists(), sorted(os.listdir(tmp_path / "unweighted"))
            rp, ci, va = bna.csr_read(str(f))
            assert va is None
            assert np.array_equal(rp, R) and np.array_equal(ci, C)
            # file layout: int Rlength, R, int Clength, C and nothing more
            assert os.path.getsize(f) == 4 * (1 + len(R) + 1 + len(C))
    assert not (tmp_path / "weighted").exists()
    out = _run("bna_cormat_u", tmp_path, tmp_path / "mask.nii", 0.5, "n", "n", "s", 2.5)
    tau, k, drop = oracle.density(oracle.cormat_packed(oracle.zscore(bolds[0])), N, 2.5)
    f = glob.glob(str(tmp_path / "unweighted" / f"s1_{N}_spa2.500%_cor*.csr"))
    assert len(f) == 1, out
    rp, ci, va = bna.csr_read(f[0])
    assert va is None and len(ci) == 2 * k
    _run("bna_cuec", tmp_path / "unweighted")
    rp, ci, _ = bna.csr_read(f[0])
    e, lam, it, conv = oracle.ec(rp, ci)
    ec = np.fromfile(f[0][:-4] + "_ec.nm", np.float32, offset=4)
    assert np.max(np.abs(ec - e)) <= 1e-5 * np.max(np.abs(e)) + 1e-6


def test_degree_tool_and_api(tmp_path, builder):
    """Degree (W/Degree/Degree/Degree.cpp:80-84): float sum of each row's
    values in column order, bit-identical; binary graphs: row lengths."""
    import torch
    b = bna.synth_bold(2000, 120, 12, 77)
    res = builder.corr_csr(torch.from_numpy(b).cuda(), mode="r_gt", value=0.3,
                           precision="bf16x3")
    g = res.numpy()
    ref = np.zeros(2000, np.float32)
    for k in range(2000):  # the reference's sequential float loop
        for v in g.val[g.row_ptr[k]:g.row_ptr[k + 1]]:
            ref[k] = np.float32(ref[k] + v)
    assert np.array_equal(builder.degree(res).cpu().numpy(), ref)
    bna.csr_write(str(tmp_path / "g.csr"), g.row_ptr, g.col_idx, g.val)
    _run("bna_degree", tmp_path)
    d = np.fromfile(tmp_path / "g_deg.nm", np.float32, offset=4)
    assert np.array_equal(d, ref)
    binres = builder.corr_csr(torch.from_numpy(b).cuda(), mode="r_gt", value=0.3,
                              precision="bf16x3", weighted=False)
    assert np.array_equal(builder.degree(binres).cpu().numpy(),
                          np.diff(g.row_ptr).astype(np.float32))



def test_modularity_tool(tmp_path):
    """Modularity tool (U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp
    main :35-162): <name>_modu.nm holds the reference's own labels as floats;
    <name>_modu.txt logs every round and, per network (the real one, then each
    random rewiring), the module count and Q."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "modularity_ref.npz"))
    R, C = g["planted300_R"], g["planted300_C"]
    bna.csr_write(str(tmp_path / "p.csr"), R, C, None)
    out = _run("bna_modularity", tmp_path, 2)
    raw = np.fromfile(tmp_path / "p_modu.nm", np.int32, count=1)
    lab = np.fromfile(tmp_path / "p_modu.nm", np.float32, offset=4)
    assert raw[0] == len(R) - 1
    assert np.array_equal(lab, g["planted300_labels"].astype(np.float32))
    log = (tmp_path / "p_modu.txt").read_text()
    _, q_o, m_o, _ = oracle.modularity(R, C)
    heads = re.findall(r"Number of Modules: (\d+),\tQ=([-\d.e+]+)", log)
    assert len(heads) == 3, log
    assert int(heads[0][0]) == m_o and abs(float(heads[0][1]) - q_o) <= 1e-5 * abs(q_o)
    # the random networks are less modular than the planted one
    assert all(float(q) < q_o for _, q in heads[1:])
    rounds = re.findall(r"Round:\t(\d+)\tnumber of nodes:\t(\d+)\t", log)
    assert rounds[0] == ("0", str(len(R) - 1)) and "Divide?: 1" in log
    assert "Save partition results as" in out
