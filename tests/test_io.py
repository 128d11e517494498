"""The map's on-disk outputs (include/se/map/io/*): meshes as PLY / VTK / OBJ with the output
transform applied, VTK point clouds, and (GPU) VTK field slices that hold getData's field values
and Map::saveMesh of a marching-cubes mesh."""
import numpy as np
import pytest


def _faces():
    rng = np.random.default_rng(0)
    return rng.uniform(0, 10, (7, 3, 3)).astype(np.float32)


def _T():
    T = np.eye(4, dtype=np.float32)
    T[:3, :3] = [[0, -1, 0], [1, 0, 0], [0, 0, 1]]
    T[:3, 3] = (1.0, 2.0, 3.0)
    return T


def test_mesh_formats(tmp_path):
    se = pytest.importorskip("supereight2_gb300")
    f, T = _faces(), _T()
    want = (f.reshape(-1, 3) @ T[:3, :3].T + T[:3, 3]).astype(np.float32)
    se.save_mesh(f, tmp_path / "m.ply", T)
    lines = (tmp_path / "m.ply").read_text().splitlines()
    assert lines[0] == "ply" and "element vertex 21" in lines and "element face 7" in lines
    body = lines[lines.index("end_header") + 1:]
    v = np.array([[float(x) for x in l.split()] for l in body[:21]], np.float32)
    assert np.allclose(v, want, atol=1e-5)
    assert body[21].split()[:4] == ["3", "0", "1", "2"] and len(body) == 28
    se.save_mesh(f, tmp_path / "m.vtk", T)
    txt = (tmp_path / "m.vtk").read_text()
    assert "DATASET POLYDATA" in txt and "POINTS 21 float" in txt and "POLYGONS 7 28" in txt
    se.save_mesh(f, tmp_path / "m.obj", T)
    obj = (tmp_path / "m.obj").read_text().splitlines()
    assert sum(l.startswith("v ") for l in obj) == 21 and sum(l.startswith("f ") for l in obj) == 7
    assert [l for l in obj if l.startswith("f ")][0] == "f 1 2 3"
    with pytest.raises(se.SeGpuError):
        se.save_mesh(f, tmp_path / "m.stl", T)


def test_supported_mesh_extensions(tmp_path):
    """mesh_io_unittest.cpp (MeshIO.hasSupportedMeshExtension): .ply, .vtk and .obj names are
    written, a bare ".ply" included; other names (an image extension, the empty name) are refused
    before any file is created."""
    se = pytest.importorskip("supereight2_gb300")
    f, T = _faces(), _T()
    for name in ("foo.ply", "bar.vtk", "bar.obj", ".ply"):
        se.save_mesh(f, tmp_path / name, T)
        assert (tmp_path / name).stat().st_size > 0
    for name in ("foo.png", ""):
        with pytest.raises(se.SeGpuError):
            se.save_mesh(f, str(tmp_path / name) if name else name, T)
    assert not (tmp_path / "foo.png").exists()


def test_mesh_face_scales(tmp_path):
    """Multi-res meshes carry a scale per face: the VTK cell data lists it, the PLY face colour
    follows it (io::save_mesh's scale_colour)."""
    se = pytest.importorskip("supereight2_gb300")
    f, T = _faces(), _T()
    sc = np.array([0, 1, 2, 3, 1, 0, 2], np.int8)
    se.save_mesh(f, tmp_path / "s.vtk", T, scales=sc)
    lines = (tmp_path / "s.vtk").read_text().splitlines()
    i = lines.index("SCALARS scale unsigned_char")
    assert [int(v) for v in lines[i + 2: i + 9]] == sc.tolist()
    assert "COLOR_SCALARS scale_colour 3" in lines
    se.save_mesh(f, tmp_path / "s.ply", T, scales=sc)
    body = (tmp_path / "s.ply").read_text().splitlines()
    faces = body[-7:]
    rgb = [tuple(l.split()[4:]) for l in faces]
    assert rgb[0] == rgb[5] and rgb[1] == rgb[4] and rgb[2] == rgb[6] and len(set(rgb)) == 4
    with pytest.raises(se.SeGpuError):
        se.save_mesh(f, tmp_path / "s.vtk", T, scales=sc[:3])


def test_point_cloud_vtk(tmp_path):
    se = pytest.importorskip("supereight2_gb300")
    p = np.arange(30, dtype=np.float32).reshape(10, 3)
    se.save_point_cloud_vtk(p, tmp_path / "p.vtk", _T())
    lines = (tmp_path / "p.vtk").read_text().splitlines()
    i = lines.index("POINTS 10 FLOAT")
    v = np.array([[float(x) for x in l.split()] for l in lines[i + 1:i + 11]], np.float32)
    assert np.allclose(v, p @ _T()[:3, :3].T + _T()[:3, 3])


@pytest.mark.gpu
def test_field_slices_and_saved_mesh(oracle, gpu, tmp_path):
    import torch
    from supereight2_gb300 import synthetic as syn
    spec, scene, poses, frames = syn.dataset("tsdf320", 3)
    args = dict(width=spec.width, height=spec.height, fx=spec.fx, fy=spec.fy, cx=spec.cx, cy=spec.cy,
                near_plane=spec.near_plane, far_plane=spec.far_plane)
    om = oracle.OracleMap(5.12, 0.02)
    gm = gpu.Map(5.12, 0.02, max_blocks=1 << 16)
    integ = gpu.MapIntegrator(gm)
    for i, (T, d) in enumerate(zip(poses, frames)):
        om.integrate_depth(d, oracle.pinhole(**args), T.astype(np.float32), i)
        integ.integrateDepth(i, torch.from_numpy(d).cuda(), gpu.PinholeCamera(**args), T.astype(np.float32))
    p_W = np.array([0.3, -0.2, 0.1], np.float32)
    gm.saveFieldSlices(tmp_path / "x.vtk", "", tmp_path / "z.vtk", p_W)
    size = gm.size
    lines = (tmp_path / "x.vtk").read_text().splitlines()
    assert f"DIMENSIONS 1 {size} {size}" in lines
    vals = np.array([float(l) for l in lines[lines.index("LOOKUP_TABLE default") + 1:] if l.strip()], np.float32)
    assert len(vals) == size * size
    # the values are getData's field: compare a sample with the oracle
    vx = int((p_W[0] + 2.56) / 0.02)
    rng = np.random.default_rng(1)
    for _ in range(200):
        y, z = rng.integers(0, size, 2)
        t, _ = om.get_data(((np.array([vx, y, z]) + 0.5) * 0.02 - 2.56).astype(np.float32))
        assert vals[z * size + y] == np.float32(t)
    assert (tmp_path / "z.vtk").exists() and not (tmp_path / "y.vtk").exists()
    gm.saveMesh(tmp_path / "mesh.ply")
    head = (tmp_path / "mesh.ply").read_text().splitlines()[:8]
    n_faces = int([l for l in head if l.startswith("element face")][0].split()[-1])
    assert n_faces == len(om.marching_cubes()) > 0
