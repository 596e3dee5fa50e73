"""Restart and output files (host code of the library, no GPU needed): the PETSc
binary Vec record the reference's monitor writes (restart1.bin, read back by
VecLoad at start-up) and legacy VTK 2.0 ASCII output."""
import numpy as np
import pytest


def test_petsc_vec_record_layout(hype, tmp_path):
    """int32 class id 1211214, int32 length, big-endian doubles; .info carries the block size"""
    v = np.random.default_rng(1).standard_normal(3 * 4 * 5 * 5)
    v[3] = -0.0
    v[7] = np.inf
    path = tmp_path / "restart1.bin"
    hype.write_petsc_vec(path, v, block_size=5)
    raw = path.read_bytes()
    assert len(raw) == 8 + 8 * v.size
    hdr = np.frombuffer(raw[:8], dtype=">i4")
    assert hdr[0] == 1211214 and hdr[1] == v.size
    body = np.frombuffer(raw[8:], dtype=">f8")
    assert np.array_equal(body.astype(np.float64).view(np.uint64), v.view(np.uint64))  # bit for bit, -0 and inf too
    assert (tmp_path / "restart1.bin.info").read_text().strip() == "-vecload_block_size 5"
    back = hype.read_petsc_vec(path, v.size)
    assert np.array_equal(back.view(np.uint64), v.view(np.uint64))


def test_petsc_vec_reader_rejects_wrong_records(hype, tmp_path):
    path = tmp_path / "x.bin"
    hype.write_petsc_vec(path, np.arange(10.0))
    assert not (tmp_path / "x.bin.info").exists()  # block size 1: no .info
    with pytest.raises(RuntimeError):
        hype.read_petsc_vec(path, 11)  # length mismatch
    path.write_bytes(np.array([1211215, 2], dtype=">i4").tobytes() + np.zeros(2, dtype=">f8").tobytes())
    with pytest.raises(RuntimeError):
        hype.read_petsc_vec(path, 2)  # not a Vec class id
    path.write_bytes(np.array([1211214, 4], dtype=">i4").tobytes() + np.zeros(2, dtype=">f8").tobytes())
    with pytest.raises(RuntimeError):
        hype.read_petsc_vec(path, 4)  # truncated
    with pytest.raises(RuntimeError):
        hype.read_petsc_vec(tmp_path / "missing.bin", 4)


def test_vtk_legacy_ascii(hype, tmp_path):
    nz, ny, nx, nc = 2, 3, 4, 5
    a = np.random.default_rng(2).standard_normal((nz, ny, nx, nc))
    path = tmp_path / "sol-00010.vtk"
    names = ["density", "x-momentum", "y-momentum", "z-momentum", "energy"]
    hype.write_vtk(path, a, h=0.25, origin=(-1.0, 0.0, 2.0), names=names)
    lines = path.read_text().splitlines()
    assert lines[0] == "# vtk DataFile Version 2.0" and lines[2] == "ASCII"
    assert lines[3] == "DATASET STRUCTURED_POINTS"
    assert lines[4] == f"DIMENSIONS {nx} {ny} {nz}"
    assert [float(t) for t in lines[5].split()[1:]] == [-0.875, 0.125, 2.125]
    assert lines[7] == f"POINT_DATA {nx * ny * nz}"
    pos = 8
    for c in range(nc):
        assert lines[pos] == f"SCALARS {names[c]} double 1" and lines[pos + 1] == "LOOKUP_TABLE default"
        vals = np.array([float(t) for t in lines[pos + 2:pos + 2 + nx * ny * nz]])
        assert np.array_equal(vals, a[..., c].ravel())  # %.17g round-trips doubles exactly
        pos += 2 + nx * ny * nz
    assert pos == len(lines)
