"""Group parity: the drop-in BoundaryClassifier against the reference's own
classification.

Every single-component fixture under tests/golden was made by running the
reference's BoundaryClassifier (taichi_lbm/BoundaryCondition.py:22-39) on the predicates
of tests/golden/make_golden.py (build_channel, build_shanchen) and recording each group's
nodes as g_<name>.  Here the same predicates, written the same way (scalar
Python over lb.mask and lb.c, so the classifier evaluates them node by node),
go through the drop-in API: the mask helpers (Mask_cricle_identify,
Mask_rectangle_identify; BoundaryCondition.py:464-475) rebuild the mask, and
each BoundarySpec is classified again.  Mask and group counts and the sorted
index sets must equal the fixture's bit for bit (the reference appends nodes
with an atomic counter, so its order carries no meaning).
"""
import numpy as np
import pytest

from tests.cases import fixture_names, load_fixture

pytestmark = pytest.mark.gpu

CASES = fixture_names()


@pytest.fixture(scope="module")
def tl(built):
    import taichi_lbm
    return taichi_lbm


def classify(tl, meta):
    """The groups of make_golden.build_channel / build_shanchen, through the
    drop-in API."""
    nx, ny = int(meta["NX"]), int(meta["NY"])
    lb = tl.LBField(meta["name"], nx, ny, 1)
    be = tl.BoundaryEngine()
    cls = tl.BoundaryClassifier((nx, ny))
    if meta.get("disc"):
        be.Mask_cricle_identify(lb, *meta["disc"])
    for r in meta.get("rects") or []:
        be.Mask_rectangle_identify(lb, *r)
    mask = lb.mask.to_numpy()

    def fluid_fn(i, j):
        return lb.mask[i, j] == 1

    def has_missing_link(i, j):
        flag = 0
        for k in range(9):
            ix2 = i - lb.c[k, 0]
            iy2 = j - lb.c[k, 1]
            if ix2 < 0 or ix2 > nx - 1 or iy2 < 0 or iy2 > ny - 1:
                flag = 1
            elif lb.mask[ix2, iy2] == -1:
                flag = 1
        return flag

    def wall_fn(i, j):
        return lb.mask[i, j] == 1 and has_missing_link(i, j) == 1

    def inside_fn(i, j):
        return lb.mask[i, j] == 1 and has_missing_link(i, j) == 0

    def inlet_fn(i, j):
        return lb.mask[i, j] == 1 and i == 0

    def outlet_fn(i, j):
        return lb.mask[i, j] == 1 and i == nx - 1

    def row_fn(jj):
        return lambda i, j2: i == 0 and j2 == jj and lb.mask[i, j2] == 1

    preds = {"fluid": fluid_fn, "periodic": fluid_fn, "stream": fluid_fn, "inside": inside_fn, "wall": wall_fn,
             "inlet": inlet_fn, "outlet": outlet_fn}
    groups = {}
    for b in meta["bcs"]:
        name = b["name"]
        if name.startswith("inlet") and name != "inlet":
            fn = row_fn(int(name[5:]))
        else:
            fn = preds[name]
        g = cls.get_group(tl.BoundarySpec(geometry_fn=fn))
        groups["g_" + name] = g.nodes
    # psi boundaries: FixedPsi on a lattice row, the open psi boundaries on
    # a row of the psi grid (-1..NX, -1..NY), nodes 0 <= i < NX
    psi_cls = tl.BoundaryClassifier((nx + 2, ny + 2), offset=(-1, -1))
    for pb in meta.get("psi_bcs", []):
        if not isinstance(pb, dict):
            continue
        row = pb["row"]
        if pb["kind"] == "fixed":
            g = cls.get_group(tl.BoundarySpec(geometry_fn=lambda i, j, r=row: (lb.mask[i, j] == 1) & (j == r)))
        else:
            g = psi_cls.get_group(tl.BoundarySpec(geometry_fn=lambda i, j, r=row: (j == r) & (i >= 0) & (i < nx)))
        groups["g_" + pb["name"]] = g.nodes
    return mask, groups


def as_sorted(nodes):
    a = np.asarray(nodes, np.int32).reshape(-1, 2)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


@pytest.mark.parametrize("name", CASES)
def test_classifier_matches_reference_groups(tl, name):
    meta, arrays = load_fixture(name)
    mask, groups = classify(tl, meta)
    assert np.array_equal(mask, arrays["mask"]), "mask differs from the reference's"
    assert set(groups) == {k for k in arrays if k.startswith("g_")}
    for k, nodes in groups.items():
        ref = arrays[k]
        assert nodes.shape[0] == ref.shape[0], f"{k}: count {nodes.shape[0]} != {ref.shape[0]}"
        assert np.array_equal(as_sorted(nodes), as_sorted(ref)), f"{k}: node set differs"
