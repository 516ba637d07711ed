"""Headless VTK export (the reference writes pyvista ImageData, evoxels/voxelfields.py:196-214):
legacy structured points, cell data in Fortran order, binary (big-endian float32) or ASCII."""

import numpy as np


def _read_legacy(path):
    raw = open(path, "rb").read()
    lines, pos = [], 0
    fields = {}
    binary = None
    while pos < len(raw):
        end = raw.index(b"\n", pos)
        line = raw[pos:end].decode()
        pos = end + 1
        lines.append(line)
        if line in ("BINARY", "ASCII"):
            binary = line == "BINARY"
        if line.startswith("CELL_DATA"):
            ncell = int(line.split()[1])
        if line.startswith("SCALARS"):
            name = line.split()[1]
            end = raw.index(b"\n", pos)   # LOOKUP_TABLE default
            pos = end + 1
            if binary:
                fields[name] = np.frombuffer(raw[pos:pos + 4 * ncell], dtype=">f4").astype(np.float32)
                pos += 4 * ncell + 1
            else:
                vals = raw[pos:].split(b"\n")[:ncell]
                fields[name] = np.array([float(v) for v in vals], dtype=np.float32)
                pos += sum(len(v) + 1 for v in vals)
    return lines, fields


def test_vtk_binary_and_ascii_roundtrip(tmp_path):
    from evoxels_gb300.voxelfields import VoxelFields
    shape = (5, 4, 3)
    vf = VoxelFields(shape, domain_size=(10.0, 4.0, 6.0))
    a = np.random.default_rng(0).random(shape)
    b = np.arange(np.prod(shape), dtype=np.float64).reshape(shape)
    vf.add_field("a", a)
    vf.add_field("b", b)
    for binary in (True, False):
        p = tmp_path / f"out_{binary}.vtk"
        vf.export_to_vtk(str(p), binary=binary)
        lines, fields = _read_legacy(str(p))
        assert "DATASET STRUCTURED_POINTS" in lines
        assert "DIMENSIONS 6 5 4" in lines
        assert "SPACING 2.0 1.0 2.0" in lines
        assert "ORIGIN 0.0 0.0 0.0" in lines   # lower cell corner: origin - spacing/2
        for name, ref in (("a", a), ("b", b)):
            np.testing.assert_array_equal(fields[name], ref.astype(np.float32).flatten(order="F"))
    p = tmp_path / "one.vtk"
    vf.export_to_vtk(str(p), field_names=["b"])
    assert list(_read_legacy(str(p))[1]) == ["b"]
