"""Host-side pieces of the headless I/O and the sparse-matrix mirror (CPU)."""

import numpy as np
import torch

from conftest import rng


def test_png_round_trip(tmp_path):
    from panopaea_gb300 import io

    img = rng(1).integers(0, 256, (7, 11, 3), dtype=np.uint8)
    p = str(tmp_path / "a.png")
    io.write_png(p, img)
    assert open(p, "rb").read()[:8] == b"\x89PNG\r\n\x1a\n"
    assert np.array_equal(io.read_png(p), img)


def test_field_dump_round_trip(tmp_path):
    from panopaea_gb300 import io

    t = torch.from_numpy(rng(2).standard_normal(5 * 6 + 6 * 4).astype(np.float64))
    p = str(tmp_path / "f.bin")
    io.save_field(p, t, "faces", (5, 4))
    back, kind, dims = io.load_field(p, device="cpu")
    assert kind == "faces" and dims == (5, 4) and torch.equal(back, t)


def test_transfer_oracle_matches_reference_formula(oracle):
    """imgproc.rs:2-5 restated in numpy (f64): the oracle agrees, and the
    image rows are flipped as png.rs:12 writes them."""
    f = np.array([[-3.0, -2.0, -1.0, 0.0], [0.5, 1.999, 2.0, 7.0], [np.nan, -0.0, 1e-9, -1e-9]])
    out = oracle.transfer_rgb8(f, -2.0, 2.0)
    v = np.clip(np.where(np.isnan(f), 2.0, f), -2.0, 2.0)
    want = np.floor((v + 2.0) / 4.0 * 255.0).astype(np.uint8)[::-1]
    assert np.array_equal(out[..., 0], want) and np.array_equal(out[..., 1], want)


def test_sparse_insert_semantics():
    """sparse.rs:63-86: columns stay sorted per row, re-inserting overwrites."""
    from panopaea_gb300.sparse import SparseMatrix

    m = SparseMatrix((3, 4))
    for (i, j, v) in [(1, 3, 1.0), (1, 0, 2.0), (0, 2, 3.0), (1, 3, 4.0), (2, 1, 5.0), (1, 1, 6.0)]:
        m.insert((i, j), v)
    rp, ci, d = m.to_csr_numpy()
    assert list(rp) == [0, 1, 4, 5]
    assert list(ci) == [2, 0, 1, 3, 1]
    assert list(d) == [3.0, 2.0, 6.0, 4.0, 5.0]
    try:
        m.insert((3, 0), 1.0)
        assert False
    except IndexError:
        pass


def test_csr_oracle(oracle):
    rp = np.array([0, 2, 2, 5])
    ci = np.array([1, 0, 0, 2, 1])
    d = np.array([2.0, 3.0, 4.0, 5.0, 6.0])
    x = np.array([1.0, 10.0, 100.0])
    assert list(oracle.csr_mul_vec(rp, ci, d, x)) == [23.0, 0.0, 564.0]
