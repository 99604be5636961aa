"""JSON mesh files (gpumesh_gb300.meshio) against the reference's own
JsonSerializer / JsonDeserializer and boundaries: a committed file written by
the reference, byte-identical output in the reference's precision, exact
round trips, and every boundary's constraint table (Box, Sphere, Tet, Shell,
Pipe) projecting as the reference's constraint objects do."""

import os

import numpy as np
import pytest

import pyoracle
import pyref

from gpumesh_gb300 import meshgen, meshio

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "tet_box_2_ref.json")
need_ref = pytest.mark.skipif(not pyref.available(), reason="reference tree not available")


def _as_reference_printed(x):
    # what the reference's `ostream << double` writes, read back
    return np.vectorize(lambda v: float("%g" % v))(x)


def test_reads_a_file_written_by_the_reference():
    raw = meshio.read_json(GOLDEN)
    src = meshgen.box_mesh(2, "tet", 0.3, 0)
    assert raw.name == "box-tet-2"
    assert np.array_equal(raw.pos, _as_reference_printed(src.pos))
    assert np.array_equal(raw.tets, src.tets) and raw.pris.shape == (0, 6) and raw.hexs.shape == (0, 8)
    assert np.array_equal(raw.cid, src.cid)
    assert np.array_equal(raw.con_kind, src.con_kind) and np.array_equal(raw.con_param, src.con_param)


@pytest.mark.parametrize("kind", ["tet", "mixed", "hex"])
def test_exact_round_trip(tmp_path, kind):
    src = meshgen.box_mesh(3, kind, 0.2, 4, gaussian=True)
    path = str(tmp_path / "m.json")
    meshio.write_json(path, src, precision="exact")
    back = meshio.read_json(path)
    for a in ("pos", "tets", "pris", "hexs", "cid", "con_kind", "con_param"):
        assert np.array_equal(getattr(back, a), getattr(src, a)), a
    assert back.name == src.name


def test_sphere_round_trip(tmp_path):
    src = meshgen.sphere_mesh(6, 0.25, 1)
    path = str(tmp_path / "s.json")
    meshio.write_json(path, src)
    back = meshio.read_json(path)
    assert np.array_equal(back.pos, src.pos) and np.array_equal(back.cid, src.cid)
    assert meshio.boundary_name(back) == "Sphere"


def test_rejects_unknown_tags_and_bad_ids(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text('{"verts": [[0,0,0]], "colour": [1]}')
    with pytest.raises(ValueError, match="unknown tag"):
        meshio.read_json(str(p))
    p.write_text('{"verts": [[0,0,0],[1,0,0],[0,1,0]], "tets": [[0,1,2,3]]}')
    with pytest.raises(ValueError, match="outside"):
        meshio.read_json(str(p))
    p.write_text('{"Boundary": "Box", "verts": [[0,0,0]], "topos": [19]}')
    with pytest.raises(ValueError, match="not a Box constraint"):
        meshio.read_json(str(p))


def test_missing_topos_and_unknown_boundary_mean_free(tmp_path):
    p = tmp_path / "free.json"
    p.write_text('{"Boundary": "Nowhere", "verts": [[0,0,0],[1,0,0],[0,1,0],[0,0,1]], "tets": [[0,1,2,3]]}')
    raw = meshio.read_json(str(p))
    assert np.array_equal(raw.cid, np.zeros(4, np.int32)) and meshio.boundary_name(raw) == "Free"


@need_ref
@pytest.mark.parametrize("case", ["tet", "mixed", "sphere"])
def test_reference_precision_output_is_byte_identical(tmp_path, case):
    if case == "sphere":
        src, boundary, name = meshgen.sphere_mesh(5, 0.25, 1), "sphere", "Sphere"
    else:
        src, boundary, name = meshgen.box_mesh(3, case, 0.2, 4, gaussian=True), "box", "Box"
    mine, theirs = str(tmp_path / "mine.json"), str(tmp_path / "ref.json")
    meshio.write_json(mine, src, boundary=name, model="m", precision="reference")
    pyref.json_write(theirs, src, boundary, "m")
    assert open(mine).read() == open(theirs).read()


@need_ref
def test_reader_agrees_with_the_reference_reader(tmp_path):
    src = meshgen.box_mesh(3, "mixed", 0.2, 4, gaussian=True)
    path = str(tmp_path / "m.json")
    meshio.write_json(path, src, precision="exact")
    ref = pyref.json_read(path)
    mine = meshio.read_json(path)
    assert ref["boundary"] == "Box" and ref["model"] == mine.name
    for a in ("pos", "cid", "tets", "pris", "hexs"):
        assert np.array_equal(ref[a], getattr(mine, a)), a


@need_ref
@pytest.mark.parametrize("boundary", ["Tet", "Shell", "Pipe", "Box", "Sphere"])
def test_boundary_tables_project_like_the_reference(boundary):
    kind, par = meshio.boundary_table(boundary)
    ids = [i for i in range(kind.shape[0]) if kind[i] != meshgen.CON_VOLUME]
    # an oracle mesh with one vertex per constraint id, projecting through it
    n = kind.shape[0]
    orc = pyoracle.OracleMesh(np.zeros((n, 3)), np.zeros((0, 4), np.uint32), np.zeros((0, 6), np.uint32),
                              np.zeros((0, 8), np.uint32), np.arange(n, dtype=np.int32), kind, par)
    rng = np.random.default_rng(7)
    pts = rng.uniform(-1.5, 1.5, (64, 3))
    for i in ids:
        theirs = pyref.boundary_project(boundary.lower(), i, pts)
        mine = np.array([orc.project(i, p) for p in pts])
        assert np.array_equal(mine, theirs), (boundary, i)
