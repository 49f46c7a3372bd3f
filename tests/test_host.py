"""Host-side logic without a GPU: the C ABI library's exports, group
classification, mask helpers and the fused-plan compiler."""
import re

import numpy as np
import pytest
import torch

from tests.cases import ROOT, fixture_names, load_fixture


def header_functions():
    src = open(f"{ROOT}/include/lbm_gb300.h").read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t)\s+(lbm_\w+)\s*\(", src, re.M)))


def test_library_exports_every_header_function(built):
    import ctypes
    from taichi_lbm import _capi
    lib = ctypes.CDLL(_capi.LIB_PATH)
    names = header_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in lbm_gb300.h but not exported"
    assert set(names) == set(_capi.EXPORTED)
    assert lib.lbm_abi_version() == 4


def test_library_reports_argument_errors(built):
    """Argument checks run before any CUDA call and set lbm_last_error."""
    import ctypes
    from taichi_lbm import _capi
    _capi.load()
    rc = _capi.load().lbm_plan_create(None, None)
    assert rc == -1 and "NULL" in _capi.last_error()
    d = _capi.LbmPlanDesc()
    d.nx, d.ny, d.pitch = 10, 10, 30  # pitch not a multiple of 32
    p = ctypes.c_void_p()
    assert _capi.load().lbm_plan_create(ctypes.byref(d), ctypes.byref(p)) == -1
    assert "pitch" in _capi.last_error()
    d.pitch, d.nodes_per_thread = 32, 3
    assert _capi.load().lbm_plan_create(ctypes.byref(d), ctypes.byref(p)) == -3


def test_classifier_vectorised_equals_scalar():
    from taichi_lbm.boundary import BoundaryClassifier, BoundarySpec, evaluate_predicate
    mask = np.ones((20, 9), np.int32)
    mask[5:8, 3:6] = -1

    def vec(i, j):
        return (mask[i, j] == 1) & ((i == 0) | (j == 8))

    def scalar(i, j):
        return mask[i, j] == 1 and (i == 0 or j == 8)

    a = evaluate_predicate(vec, 20, 9)
    b = evaluate_predicate(scalar, 20, 9)  # raises on arrays -> node by node
    assert np.array_equal(a, b) and a.sum() == 9 + 20 - 1
    cls = BoundaryClassifier((20, 9), device=torch.device("cpu"))
    g = cls.get_group(BoundarySpec(geometry_fn=scalar))
    assert g.count[None] == a.sum()
    assert np.array_equal(g.nodes, np.argwhere(a.T)[:, ::-1])  # row-major in memory: j, then i
    gp = BoundaryClassifier((22, 11), offset=(-1, -1), device=torch.device("cpu")).get_group(
        BoundarySpec(geometry_fn=lambda i, j: (i == -1) | (j == 9)))
    assert gp.nodes[:, 0].min() == -1 and gp.count[None] == 11 + 22 - 1


@pytest.mark.parametrize("name", ["cyl_bgk_f32", "contraction_pl_trt_n05_f32"])
def test_host_mask_helpers_bit_exact(name):
    """BoundaryEngine.Mask_*_identify on the host (f32 arithmetic) gives the
    reference's mask exactly."""
    from taichi_lbm.boundary import BoundaryEngine
    from taichi_lbm.fields import MaskField
    meta, arrays = load_fixture(name)

    class FakeField:
        NX, NY = meta["NX"], meta["NY"]
        mask = MaskField(meta["NX"], meta["NY"])
    lb = FakeField()
    be = BoundaryEngine()
    if meta.get("disc"):
        be.Mask_cricle_identify(lb, *meta["disc"])
    for r in meta.get("rects", []):
        be.Mask_rectangle_identify(lb, *r)
    assert np.array_equal(lb.mask.arr, arrays["mask"])


def links_from_mask(mask):
    """LBField.neighbor in bit form, as lbm_neighbor_classify computes it."""
    nx, ny = mask.shape
    c = np.array([[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1], [-1, -1], [1, -1]])
    links = np.zeros((nx, ny), np.int64)
    for i in range(nx):
        for j in range(ny):
            if mask[i, j] == -1:
                continue
            b = 0x8000
            for k in range(9):
                i2, j2 = i - c[k, 0], j - c[k, 1]
                if 0 <= i2 < nx and 0 <= j2 < ny and mask[i2, j2] != -1:
                    b |= 1 << k
            links[i, j] = b
    return links


def items_from_fixture(meta, arrays):
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import BoundaryItem
    kinds = {"fluid": A.BC_FLUID, "periodic": A.BC_PERIODIC, "inside": A.BC_INSIDE,
             "bounceback": A.BC_BOUNCEBACK, "velocity_eq": A.BC_VELOCITY_EQ,
             "velocity_neem": A.BC_VELOCITY_NEEM, "velocity_bb": A.BC_VELOCITY_BB,
             "pressure_neem": A.BC_PRESSURE_NEEM, "pressure_abc": A.BC_PRESSURE_ABC,
             "open_neumann": A.BC_OPEN_NEUMANN, "open_conv1": A.BC_OPEN_CONV1,
             "open_extrap": A.BC_OPEN_EXTRAP}
    items = []
    for b in meta["bcs"]:
        nd = arrays["g_" + b["name"]]
        vel = None
        if "velocity" in b:
            vel = np.tile(np.asarray(b["velocity"], np.float32), (nd.shape[0], 1))
        items.append(BoundaryItem(kinds[b["kind"]], nd, b.get("direction", 0), b.get("rho", 0.0), vel,
                                  b["name"]))
    return items


def test_plan_compiler_cylinder_fixture():
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import compile_plan
    meta, arrays = load_fixture("cyl_bgk_f32")
    nx, ny = meta["NX"], meta["NY"]
    links = links_from_mask(arrays["mask"])
    fluid = arrays["g_fluid"]
    cp = compile_plan(nx, ny, fluid, links, items_from_fixture(meta, arrays), 4)
    code = cp.code.astype(np.int64)
    active = (code & A.CODE_ACTIVE) != 0
    assert active.sum() == fluid.shape[0]
    assert not active[arrays["mask"] == -1].any()
    # bounce bits exactly on the missing links of the wall group
    wall = arrays["g_wall"]
    for i, j in wall:
        for k in range(1, 9):
            assert bool(code[i, j] & (1 << (k - 1))) == (not (links[i, j] >> k) & 1)
    # 20 single-node parabolic inlet boundaries merge into one instance
    kinds = [ins["kind"] for ins in cp.instances]
    assert kinds == [A.BC_VELOCITY_EQ, A.BC_PRESSURE_NEEM]
    assert cp.bc_vel is not None and cp.bc_vel[0, 0].max() > 0.04
    # PressureNEEM reads moments at the outlet node and at x - 1
    save = (code & A.CODE_SAVE) != 0
    assert save[nx - 1].sum() == ny and save[nx - 2].sum() == ny and save.sum() == 2 * ny
    # interior segments are plain: only edge/cylinder rows' segments are flagged
    assert cp.seg_flags.shape == (ny, 1)
    assert cp.seg_flags.all()  # 40 nodes per row, one 128-wide segment holding the edges


def test_plan_compiler_refusals():
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import BoundaryItem, UnsupportedComposition, compile_plan
    nx, ny = 8, 6
    mask = np.ones((nx, ny), np.int32)
    links = links_from_mask(mask)
    allnodes = np.argwhere(mask == 1).astype(np.int32)
    edge = allnodes[(allnodes[:, 0] == 0) | (allnodes[:, 0] == nx - 1) | (allnodes[:, 1] == 0)
                    | (allnodes[:, 1] == ny - 1)]
    inlet = allnodes[allnodes[:, 0] == 0]
    fl = BoundaryItem(A.BC_FLUID, allnodes, name="fluid")
    # no stream carrier
    with pytest.raises(UnsupportedComposition, match="not covered"):
        compile_plan(nx, ny, allnodes, links, [fl], 4)
    # InsideBoundary over nodes with missing links reads outside the lattice
    with pytest.raises(UnsupportedComposition, match="outside the lattice"):
        compile_plan(nx, ny, allnodes, links, [fl, BoundaryItem(A.BC_INSIDE, allnodes, name="in")], 4)
    # a rewrite boundary applied before the carrier that overwrites it
    eq = BoundaryItem(A.BC_VELOCITY_EQ, inlet, 3, 0, np.zeros((inlet.shape[0], 2)), "eq")
    with pytest.raises(UnsupportedComposition, match="before a stream carrier"):
        compile_plan(nx, ny, allnodes, links,
                     [fl, eq, BoundaryItem(A.BC_PERIODIC, allnodes, name="p")], 4)
    # NEEM reading a neighbour an earlier boundary rewrote
    col1 = allnodes[allnodes[:, 0] == 1]
    eq1 = BoundaryItem(A.BC_VELOCITY_EQ, col1, 3, 0, np.zeros((col1.shape[0], 2)), "eq1")
    neem = BoundaryItem(A.BC_VELOCITY_NEEM, inlet, 3, 0, np.zeros((inlet.shape[0], 2)), "neem")
    with pytest.raises(UnsupportedComposition, match="already rewrote"):
        compile_plan(nx, ny, allnodes, links,
                     [fl, BoundaryItem(A.BC_PERIODIC, allnodes, name="p"), eq1, neem], 4)
    # the supported order compiles, and wall bounce bits follow the last carrier
    cp = compile_plan(nx, ny, allnodes, links,
                      [fl, BoundaryItem(A.BC_PERIODIC, allnodes, name="p"),
                       BoundaryItem(A.BC_BOUNCEBACK, edge, name="w"), eq], 4)
    assert (cp.code[0, 0] & 0xFF) != 0 and (cp.code[3, 3] & 0xFF) == 0



def test_plan_compiler_in_place_checks():
    """The in-place step pairs each node's read and write locations: a link
    cut by bounce-back on one side only, or a colliding node streaming from a
    node outside the collision group, is refused; a channel walled on every
    edge compiles and lists the nodes its NEEM outlet reads."""
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import BoundaryItem, UnsupportedComposition, compile_plan
    nx, ny = 8, 6
    mask = np.ones((nx, ny), np.int32)
    links = links_from_mask(mask)
    allnodes = np.argwhere(mask == 1).astype(np.int32)
    fl = BoundaryItem(A.BC_FLUID, allnodes, name="fluid")
    per = BoundaryItem(A.BC_PERIODIC, allnodes, name="p")
    bottom = allnodes[allnodes[:, 1] == 0]
    # bottom row bounces back what the (periodic) top row streams to it
    with pytest.raises(UnsupportedComposition, match="one side only"):
        compile_plan(nx, ny, allnodes, links, [fl, per, BoundaryItem(A.BC_BOUNCEBACK, bottom, name="w")], 4,
                     in_place=True)
    # the same composition is fine for the ping-pong step
    compile_plan(nx, ny, allnodes, links, [fl, per, BoundaryItem(A.BC_BOUNCEBACK, bottom, name="w")], 4)
    # a colliding node streaming from a node outside the collision group
    some = allnodes[allnodes[:, 0] != 3]
    with pytest.raises(UnsupportedComposition, match="outside the collision group"):
        compile_plan(nx, ny, some, links, [BoundaryItem(A.BC_FLUID, some, name="fluid"),
                                           BoundaryItem(A.BC_PERIODIC, some, name="p")], 4, in_place=True)
    # walls on every edge (both sides of every wrapped link cut) with a NEEM outlet
    edge = allnodes[(allnodes[:, 0] == 0) | (allnodes[:, 0] == nx - 1) | (allnodes[:, 1] == 0)
                    | (allnodes[:, 1] == ny - 1)]
    outlet = allnodes[allnodes[:, 0] == nx - 1]
    neem = BoundaryItem(A.BC_PRESSURE_NEEM, outlet, 1, 1.0, None, "out")
    ext = BoundaryItem(A.BC_OPEN_EXTRAP, allnodes[allnodes[:, 0] == 0], 3, 0.0, None, "ext")
    cp = compile_plan(nx, ny, allnodes, links, [fl, per, BoundaryItem(A.BC_BOUNCEBACK, edge, name="w"), neem, ext],
                      4, in_place=True)
    want = sorted({(nx - 2, j) for j in range(ny)} | {(1, j) for j in range(ny)} | {(2, j) for j in range(ny)},
                  key=lambda t: (t[1], t[0]))
    assert [tuple(t) for t in cp.read_sites.tolist()] == want
    assert compile_plan(nx, ny, allnodes, links, [fl, per], 4, in_place=True).read_sites.shape == (0, 2)

def test_segment_flags_mark_only_special_segments():
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import BoundaryItem, compile_plan
    nx, ny = 300, 4  # three 128-node segments per row at 4 nodes per thread
    mask = np.ones((nx, ny), np.int32)
    links = links_from_mask(mask)
    nodes = np.argwhere(mask == 1).astype(np.int32)
    cp = compile_plan(nx, ny, nodes, links, [BoundaryItem(A.BC_FLUID, nodes, name="f"),
                                             BoundaryItem(A.BC_PERIODIC, nodes, name="p")], 4)
    assert cp.seg_flags.shape == (ny, 3) and cp.seg_flags.sum() == 0
    assert (cp.code == A.CODE_ACTIVE).all()


@pytest.mark.parametrize("V", [2, 4, 8])
def test_lane_mask_and_lane_list_cover_exactly_the_special_nodes(V):
    """Bit l of lane_mask[y, seg] is set exactly when one of lane l's V nodes is
    not plain (bounce-back link, boundary program, saved moments, outside the
    collision group); the lane list holds the set bits as (y * nseg + seg) * 32
    + l; a segment's flag is nonzero exactly when some bit of its mask is set.
    389 columns leave a partial last segment at every V."""
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import BoundaryItem, compile_plan
    nx, ny = 389, 12
    mask = np.ones((nx, ny), np.int32)
    mask[100:110, 4:8] = -1  # a solid block
    links = links_from_mask(mask)
    fluid = np.argwhere(mask == 1).astype(np.int32)
    c = [(0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, 1), (-1, -1), (1, -1)]
    missing = np.zeros((nx, ny), bool)
    for k in range(1, 9):
        cx, cy = c[k]
        src = np.pad(mask == 1, 1, constant_values=False)[1 - cx:1 - cx + nx, 1 - cy:1 - cy + ny]
        missing |= ~src
    wall = np.argwhere((mask == 1) & missing).astype(np.int32)
    cp = compile_plan(nx, ny, fluid, links, [BoundaryItem(A.BC_FLUID, fluid, name="f"),
                                             BoundaryItem(A.BC_PERIODIC, fluid, name="p"),
                                             BoundaryItem(A.BC_BOUNCEBACK, wall, name="w")], V)
    nseg = -(-nx // (32 * V))
    lm = np.asarray(cp.lane_mask, np.uint32).reshape(ny, nseg)
    plain = cp.code == A.CODE_ACTIVE  # (nx, ny)
    want = np.zeros((ny, nseg), np.uint64)
    for y in range(ny):
        for x in range(nx):
            if not plain[x, y]:
                seg, lane = divmod(x // V, 32)
                want[y, seg] |= np.uint64(1) << np.uint64(lane)
    assert np.array_equal(lm.astype(np.uint64), want)
    ys, segs = np.nonzero(lm)
    expect = [((y * nseg + s) * 32 + l) for y, s in zip(ys, segs) for l in range(32) if (lm[y, s] >> l) & 1]
    assert sorted(np.asarray(cp.lanes).tolist()) == sorted(expect)
    assert np.array_equal(np.asarray(cp.seg_flags).reshape(ny, nseg) != 0, lm != 0)


def _aa_emulation(nx, ny, steps, seed=3):
    """Ping-pong and in-place (AA-pattern) steps emulated in numpy on a channel
    periodic in x with solid rows at y = 0 and y = ny - 1 (bounce-back from
    them), with an arbitrary per-node 'collision'; returns both states."""
    cx = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
    cy = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
    opp = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])
    active = np.ones((nx, ny), bool)
    active[:, 0] = active[:, ny - 1] = False
    bounce = np.zeros((9, nx, ny), bool)  # link k of x comes from a solid node
    for k in range(1, 9):
        bounce[k] = active & ~np.roll(active, (cx[k], cy[k]), axis=(0, 1))
    rng = np.random.default_rng(seed)
    state0 = rng.random((9, nx, ny))
    perm = np.array([0, 5, 2, 7, 4, 1, 6, 3, 8])

    def collide(f):  # any deterministic function of the node's nine values
        return 0.5 * f[perm] + 0.25 * f.sum(axis=0, keepdims=True) / 9.0

    def pulled(P):
        f = np.empty_like(P)
        for k in range(9):
            f[k] = np.where(bounce[k], P[opp[k]], np.roll(P[k], (cx[k], cy[k]), axis=(0, 1)))
        return f

    P = state0.copy()
    for _ in range(steps):  # ping-pong: pull, collide, store at the node
        post = collide(pulled(P))
        P = np.where(active[None], post, P)
    A = state0.copy()
    for s in range(steps):
        if s % 2 == 0:  # phase A: pull; write f*_opp(k) where f_k was read
            post = collide(pulled(A))
            out = A.copy()
            for k in range(9):
                val = post[opp[k]]
                # bounced links: read and written at the node itself, slot opp(k)
                out[opp[k]] = np.where(active & bounce[k], val, out[opp[k]])
                # streamed links: slot k of x - c_k
                moved = np.roll(np.where(active & ~bounce[k], val, np.nan), (-cx[k], -cy[k]), axis=(0, 1))
                out[k] = np.where(np.isnan(moved), out[k], moved)
            A = out
        else:  # phase B: f_k at slot opp(k) of the node, f*_k to slot k
            post = collide(A[opp])
            A = np.where(active[None], post, A)
    if steps % 2 == 1:  # swap each streamed pair (slot k of x, slot opp(k) of x + c_k) back
        out = A.copy()
        for k in (1, 2, 5, 6):
            tgt_active = np.roll(active, (-cx[k], -cy[k]), axis=(0, 1))
            tgt_bounce = np.roll(bounce[k], (-cx[k], -cy[k]), axis=(0, 1))
            pair = active & tgt_active & ~tgt_bounce
            other = np.roll(A[opp[k]], (-cx[k], -cy[k]), axis=(0, 1))
            out[k] = np.where(pair, other, A[k])
            back = np.roll(np.where(pair, A[k], np.nan), (cx[k], cy[k]), axis=(0, 1))
            out[opp[k]] = np.where(np.isnan(back), out[opp[k]], back)
        A = out
    return P, A


@pytest.mark.parametrize("steps", [1, 2, 5, 8])
def test_in_place_layout_algebra(steps):
    """The in-place step's two phases and the swap after an odd run leave the
    buffer holding exactly the ping-pong state (emulated in numpy: reads,
    writes and bounce-back links as the kernels do them)."""
    P, A = _aa_emulation(12, 7, steps)
    assert np.array_equal(P, A)


def test_fixtures_compile_in_place():
    """Every non-Shan-Chen fixture composition passes the in-place checks, and
    its read sites are exactly the neighbours its NEEM and open boundaries read."""
    from taichi_lbm import _capi as A
    from taichi_lbm._plan import READS, compile_plan
    cx = (0, 1, 0, -1, 0, 1, -1, -1, 1)
    cy = (0, 0, 1, 0, -1, 1, 1, -1, -1)
    checked = 0
    for name in fixture_names():
        meta, arrays = load_fixture(name)
        if meta.get("sc"):
            continue
        nx, ny = meta["NX"], meta["NY"]
        items = items_from_fixture(meta, arrays)
        cp = compile_plan(nx, ny, arrays["g_fluid"], links_from_mask(arrays["mask"]), items, 4, in_place=True)
        want = set()
        for it in items:
            if it.kind not in READS or it.nodes.size == 0:
                continue
            _, _, x2_f, x3_f = READS[it.kind]
            for d, on in ((1, x2_f), (2, x3_f)):
                if on:
                    want |= {(int(i) - d * cx[it.direction], int(j) - d * cy[it.direction]) for i, j in it.nodes}
        got = [tuple(t) for t in cp.read_sites.tolist()]
        assert got == sorted(want, key=lambda t: (t[1], t[0])), name
        checked += 1
    assert checked >= 16
