"""The reference's derivative tests 1.1-1.5 as a protocol over a renderer.

src/tests.cpp:31-107 (test_base_derivatives), :491-637 (finDiff_param,
test_fin_diff, test_derivatives) and :681-760 (PrintAndCompareGradients):

  * scenes and camera: the fixture `fd_tests1_scenes`, written by the
    reference's own src/scenes.cpp through ref_driver (scn03 triangle,
    scn05 pyramid, scn09 textured sphere; camera at z = 3, 45 degrees,
    256 x 256), 16 samples per pixel;
  * gradient: d_render of the initial scene with the adjoint 2(I - T) and
    W*H edge samples (tests.cpp:655-664);
  * finite differences: forward, h = 2/W for positions, 0.1 for colours and
    texels; per coordinate the change of sum over pixels and channels of
    (I - T)^2, divided by h (finDiff_param);
  * coordinates: the test binary's own -- every vertex of meshes with at
    most 100; for the sphere of 1.3, 100 of its vertices, and for 1.5, 250
    texels with all channels, as the binary draws them from the C library's
    rand() (recorded in the fixture by ref_driver);
  * error: sum |g - fd| / sum (|g| + |fd|) over the tested coordinates of a
    block; pass below 0.5 (positions, colours) and 0.01 (texture).

`backend` renders and differentiates: render(scene) -> float32 image (H*W*3)
and d_render(scene, adjoint) -> (gradient vector, layout row (vertices,
instances, pos, col, tex offsets, ...)).
"""
import numpy as np

from diffrender_tutorials_gb300.scene import CamInfo, Scene, Texture, TriangleMesh
from fixtures import load

W = H = 256
SPP = 16
SILHOUETTE, VERTEX_COLOR, TEXTURE_COLOR = 1, 2, 3
# test number -> (shading model, vertices tested at most, texels tested)
CASES = {1: (SILHOUETTE, 100, 0), 2: (SILHOUETTE, 100, 0), 3: (SILHOUETTE, 100, 0), 4: (VERTEX_COLOR, 100, 0),
         5: (TEXTURE_COLOR, 0, 250)}
PASS = {"pos": 0.5, "color": 0.5, "texture": 0.01}  # TESTER_FIN_DIFF_PASS, TESTER_FIN_DIFF_TEXTURE_PASS


def _mesh(d, p):
    get = lambda k: d.get(p + k)  # noqa: E731
    tex = []
    if p + "tex" in d:
        w, h, c = (int(x) for x in d[p + "tex_shape"])
        tex = [Texture(w, h, c, d[p + "tex"].copy())]
    return TriangleMesh(get("vertices").copy(), get("indices").copy(), colors=get("colors"), tc=get("tc"),
                        normals=get("normals"), tangents=get("tangents"), textures=tex)


def problem(case):
    d = load("fd_tests1_scenes")
    scenes = []
    for which in ("initial", "target"):
        s = Scene()
        s.add_mesh(_mesh(d, f"out.t1{case}.{which}."))
        scenes.append(s)
    cam = CamInfo(world_view=d["out.cam.worldview"], proj=d["out.cam.proj"], width=W, height=H)
    return scenes[0], scenes[1], cam


def run(backend, case, texels=None, central=False):
    """Errors of the case's blocks: {'pos', 'color', 'texture'} (None where
    the case tests nothing), as PrintAndCompareGradients returns them, and
    the number of tested coordinates whose difference is not zero
    ('nonzero').  texels: other texels than the test's own; central:
    central differences (L(+h) - L(-h)) / 2h instead of forward ones."""
    mode, max_v, max_t = CASES[case]
    init, target, _ = problem(case)
    tgt = backend.render(target)
    org = backend.render(init)
    adj = (2.0 * (org.astype(np.float32) - tgt.astype(np.float32))).astype(np.float32)
    g, lay = backend.d_render(init, adj)
    nv, pos, col, tex = int(lay[0]), int(lay[2]), int(lay[3]), int(lay[4])
    mse0 = ((org.astype(np.float32) - tgt.astype(np.float32)) ** 2).astype(np.float32)
    d = load("fd_tests1_scenes")
    test_vertices = d[f"out.t1{case}.test_vertices"]
    test_texels = d.get(f"out.t1{case}.test_texels", np.zeros(0, np.int32)) if texels is None else texels

    def loss_change(modify, delta):
        s = init.copy()
        modify(s.meshes[0], delta)
        img = backend.render(s)
        return ((img.astype(np.float32) - tgt.astype(np.float32)) ** 2).astype(np.float32) - mse0

    def fd(modify, delta):
        if central:
            diff = (loss_change(modify, delta) - loss_change(modify, -delta)) / np.float32(2 * delta)
        else:
            diff = loss_change(modify, delta) / np.float32(delta)
        return float(np.sum(diff, dtype=np.float64))

    out = {"pos": None, "color": None, "texture": None}
    pairs = {"pos": [], "color": [], "texture": []}
    dpos = 2.0 / W
    assert len(test_vertices) <= max_v and (texels is not None or len(test_texels) <= max_t)
    for i in test_vertices:
        i = int(i)
        for k in range(3):
            def mv(m, dlt, i=i, k=k):
                v = m.vertices.reshape(-1, 3)
                v[i, k] = np.float32(v[i, k] + np.float32(dlt))
            pairs["pos"].append((g[pos + 3 * i + k], fd(mv, dpos)))
        if mode == VERTEX_COLOR and col >= 0:
            for k in range(3):
                def mc(m, dlt, i=i, k=k):
                    c = m.colors.reshape(-1, 3)
                    c[i, k] = np.float32(c[i, k] + np.float32(dlt))
                pairs["color"].append((g[col + 3 * i + k], fd(mc, 0.1)))
    if max_t and tex >= 0:
        t0 = init.meshes[0].textures[0]
        for p in test_texels:
            for ch in range(t0.channels):
                off = int(p) * t0.channels + ch

                def mt(m, dlt, off=off):
                    m.textures[0].data[off] = np.float32(m.textures[0].data[off] + np.float32(dlt))
                pairs["texture"].append((g[tex + off], fd(mt, 0.1)))
    out["nonzero"] = 0
    for key, pr in pairs.items():
        if pr:
            a = np.array(pr, np.float64)
            out[key] = float(np.abs(a[:, 0] - a[:, 1]).sum() / (1e-12 + np.abs(a).sum()))
            out["nonzero"] += int(np.count_nonzero(a[:, 1]))
    return out


class OracleBackend:
    """The oracle (bit-exact with the reference's CPU renderer on these models)."""

    def __init__(self, mode):
        import pyoracle as O
        self.O, self.mode = O, mode
        self.cam = problem(1)[2]

    def render(self, scene):
        return self.O.render(scene, [self.cam], self.mode, SPP)

    def d_render(self, scene, adj):
        g = self.O.d_render(scene, [self.cam], self.mode, SPP, adj, W * H)
        lay, _ = self.O.dscene_layout(scene, self.mode, [0])
        return g, np.asarray(lay).reshape(-1)


class GpuBackend:
    """The GPU renderer through the C ABI (commit before every render);
    bruteforce: the reference's triangle loop instead of the hierarchy."""

    def __init__(self, mode, bruteforce=False):
        import diffrender_tutorials_gb300 as D
        from diffrender_tutorials_gb300 import native as N
        self.D = D
        self.r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(mode), SPP))
        self.r.set_option(N.OPT_TRACE_BRUTEFORCE, int(bruteforce))
        self.cam = problem(1)[2]

    def render(self, scene):
        self.r.commit(scene)
        return self.r.render(scene, [self.cam]).reshape(-1)

    def d_render(self, scene, adj):
        self.r.commit(scene)
        ds = self.D.DScene(self.r, [0])
        self.r.d_render(scene, [self.cam], adj, W * H, ds)
        return ds.data.copy(), np.asarray(ds.layout[0])
