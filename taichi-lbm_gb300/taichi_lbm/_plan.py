"""Compile a reference step composition into the fused kernel's node codes.

Pure host logic (numpy), no CUDA.  Input: the lattice size, the collision
group, the neighbor table in bit form and the ordered boundary list of a
BoundaryEngine (taichi_lbm/BoundaryCondition.py:477-483 applies them in
insertion order).  Output: one uint16 code per node (bounce bits, collide
flag, saved-moments flag, boundary program id), the per-segment fast-path
flags, the merged boundary instances and programs, and per-node boundary
velocities.

Semantics reproduced (reference step: moments, collision into f2, then every
boundary in order, each reading and writing f and the moment fields):

* A stream carrier (PeriodicAllBoundary, InsideBoundary, BounceBackWall)
  rewrites all nine populations of its nodes from f2, so a node's last
  carrier alone defines its post-stream populations: periodic -> pull with
  wrap-around, bounce-back -> pull where neighbor != -1 else f2[x][opp k],
  inside -> pull (a missing link is an out-of-range read in the reference and
  is refused).
* Rewrite boundaries that follow the node's last carrier are applied in
  order as the node's program.
* A boundary that reads f or moments of another node (NEEM, ABC, open
  boundaries) reads the start-of-step moments and the post-stream
  populations; compositions where an earlier boundary in the same step has
  already modified those values are refused, as are reads outside the
  lattice.

Anything refused raises UnsupportedComposition with the reason; the caller
can still run the same composition through the per-stage kernels.
"""
import numpy as np

from . import _capi as A

MOMENT_WRITERS = {A.BC_VELOCITY_EQ, A.BC_VELOCITY_NEEM, A.BC_PRESSURE_ABC, A.BC_PRESSURE_NEEM,
                  A.BC_OPEN_NEUMANN, A.BC_OPEN_CONV1}
# boundary kind -> (reads moments at self, reads moments at x2, reads f at x2, reads f at x3)
READS = {
    A.BC_VELOCITY_BB: (True, False, False, False),
    A.BC_VELOCITY_EQ: (False, False, False, False),
    A.BC_VELOCITY_NEEM: (False, True, True, False),
    A.BC_PRESSURE_ABC: (True, True, False, False),
    A.BC_PRESSURE_NEEM: (True, True, True, False),
    A.BC_OPEN_NEUMANN: (False, False, True, False),
    A.BC_OPEN_CONV1: (False, True, True, False),
    A.BC_OPEN_EXTRAP: (False, False, True, True),
}
VELOCITY_KINDS = {A.BC_VELOCITY_BB, A.BC_VELOCITY_EQ, A.BC_VELOCITY_NEEM}
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])


class UnsupportedComposition(ValueError):
    """The fused kernel cannot reproduce this step composition exactly."""


class BoundaryItem:
    """One boundary of the ordered list, in plain data."""

    def __init__(self, kind, nodes, direction=0, rho_value=0.0, velocity=None, name=""):
        self.kind = int(kind)
        self.nodes = np.asarray(nodes, np.int32).reshape(-1, 2)
        self.direction = int(direction or 0)
        self.rho_value = float(rho_value or 0.0)
        self.velocity = None if velocity is None else np.asarray(velocity, np.float32).reshape(-1, 2)
        self.name = name


class CompiledPlan:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def _members(nx, ny, nodes):
    m = np.zeros(nx * ny, bool)
    if nodes.size:
        m[nodes[:, 0].astype(np.int64) * ny + nodes[:, 1]] = True
    return m.reshape(nx, ny)


def compile_plan(nx, ny, collision_nodes, links, items, nodes_per_thread, in_place=False):
    """links: (nx, ny) int array, LBField.neighbor in bit form (bit k: link k
    has a source; bit 15: node classified).  in_place: also check that the
    in-place (AA-pattern) step can run the composition and list the nodes
    whose post-stream populations boundary programs read (read_sites)."""
    V = int(nodes_per_thread)
    active = _members(nx, ny, np.asarray(collision_nodes, np.int32).reshape(-1, 2))
    carrier = np.full(nx * ny, -1, np.int32)  # flat views, scattered by linear index
    carrier_kind = np.zeros(nx * ny, np.int32)
    covered = np.zeros(nx * ny, bool)
    rewrites = []
    for idx, it in enumerate(items):
        nd = it.nodes
        if nd.size and (nd.min(axis=0) < 0).any() | (nd[:, 0].max() >= nx) | (nd[:, 1].max() >= ny):
            raise UnsupportedComposition(f"boundary '{it.name}' has nodes outside the lattice")
        if it.kind == A.BC_FLUID:
            continue
        lin = nd[:, 0].astype(np.int64) * ny + nd[:, 1]
        covered[lin] = True
        if it.kind in (A.BC_PERIODIC, A.BC_INSIDE, A.BC_BOUNCEBACK):
            carrier[lin] = idx
            carrier_kind[lin] = it.kind
        elif it.kind in READS:
            rewrites.append(idx)
        else:
            raise UnsupportedComposition(f"boundary '{it.name}' (kind {it.kind}) has no fused form")
    carrier = carrier.reshape(nx, ny)
    carrier_kind = carrier_kind.reshape(nx, ny)
    covered = covered.reshape(nx, ny)

    if (active & (carrier < 0)).any():
        i, j = np.argwhere(active & (carrier < 0))[0]
        raise UnsupportedComposition(f"colliding node ({i}, {j}) is not covered by any stream "
                                     "carrier (its populations would not be streamed)")
    if (covered & ~active).any():
        i, j = np.argwhere(covered & ~active)[0]
        raise UnsupportedComposition(f"node ({i}, {j}) is in a boundary group but not in the "
                                     "collision group")

    # --- bounce bits from each node's last carrier: bit k-1 of the code is set
    # when link k has no source (bit k of the neighbor bits clear)
    code = np.zeros((nx, ny), np.int64)
    code[active] |= A.CODE_ACTIVE
    links = np.asarray(links, np.int64)
    bb = active & (carrier_kind == A.BC_BOUNCEBACK)
    ins = active & (carrier_kind == A.BC_INSIDE)
    if ((bb | ins) & ((links & 0x8000) == 0)).any():
        i, j = np.argwhere((bb | ins) & ((links & 0x8000) == 0))[0]
        raise UnsupportedComposition(f"node ({i}, {j}) streams through the neighbor table but "
                                     "was never classified (call neighbor_classify after the mask)")
    missing_bits = (~links >> 1) & 0xFF
    if (ins & (missing_bits != 0)).any():
        i, j = np.argwhere(ins & (missing_bits != 0))[0]
        k = int(np.flatnonzero([(missing_bits[i, j] >> b) & 1 for b in range(8)])[0]) + 1
        raise UnsupportedComposition(f"InsideBoundary node ({i}, {j}) has no source on link "
                                     f"{k}: the reference reads outside the lattice there")
    code |= np.where(bb, missing_bits, 0)

    # --- rewrite boundaries: ordering checks, reads, saves
    member = {idx: _members(nx, ny, items[idx].nodes) for idx in rewrites}
    f_modified_before = np.zeros((nx, ny), bool)
    mom_modified_before = np.zeros((nx, ny), bool)
    save = np.zeros((nx, ny), bool)
    for idx in rewrites:
        it = items[idx]
        nd = it.nodes
        if nd.size == 0:
            continue
        if (carrier[nd[:, 0], nd[:, 1]] > idx).any():
            raise UnsupportedComposition(f"boundary '{it.name}' is applied before a stream carrier "
                                         "that overwrites its nodes")
        if it.direction not in (1, 2, 3, 4):
            raise UnsupportedComposition(f"boundary '{it.name}' needs direction 1..4")
        self_m, x2_m, x2_f, x3_f = READS[it.kind]
        dx, dy = CX[it.direction], CY[it.direction]
        x2 = nd - np.array([dx, dy], np.int32)
        x3 = nd - 2 * np.array([dx, dy], np.int32)
        for name, pts, need in (("x2", x2, x2_m or x2_f), ("x3", x3, x3_f)):
            if not need:
                continue
            if ((pts[:, 0] < 0) | (pts[:, 0] >= nx) | (pts[:, 1] < 0) | (pts[:, 1] >= ny)).any():
                raise UnsupportedComposition(f"boundary '{it.name}' reads a neighbour outside the lattice")
            if not active[pts[:, 0], pts[:, 1]].all():
                raise UnsupportedComposition(f"boundary '{it.name}' reads a non-colliding neighbour")
            if member[idx][pts[:, 0], pts[:, 1]].any():
                raise UnsupportedComposition(f"boundary '{it.name}' reads nodes of its own group "
                                             "(order-dependent in the reference)")
            if f_modified_before[pts[:, 0], pts[:, 1]].any() and (x2_f or x3_f):
                raise UnsupportedComposition(f"boundary '{it.name}' reads populations an earlier "
                                             "boundary already rewrote in the same step")
        if x2_m:
            if mom_modified_before[x2[:, 0], x2[:, 1]].any():
                raise UnsupportedComposition(f"boundary '{it.name}' reads moments an earlier "
                                             "boundary already rewrote in the same step")
            save[x2[:, 0], x2[:, 1]] = True
        if self_m:
            if mom_modified_before[nd[:, 0], nd[:, 1]].any():
                raise UnsupportedComposition(f"boundary '{it.name}' reads moments an earlier "
                                             "boundary already rewrote in the same step")
            save[nd[:, 0], nd[:, 1]] = True
        f_modified_before |= member[idx]
        if it.kind in MOMENT_WRITERS:
            mom_modified_before |= member[idx]

    # --- merge consecutive same-kind boundaries with disjoint groups
    instances = []  # dicts: kind, direction, rho_value, members (list of idx)
    for idx in rewrites:
        it = items[idx]
        if it.nodes.size == 0:
            continue
        last = instances[-1] if instances else None
        if (last is not None and last["kind"] == it.kind and last["direction"] == it.direction
                and last["rho_value"] == it.rho_value and last["last_idx"] == _prev_rewrite(rewrites, idx)
                and not (last["mask"] & member[idx]).any()):
            last["members"].append(idx)
            last["mask"] |= member[idx]
            last["last_idx"] = idx
        else:
            instances.append({"kind": it.kind, "direction": it.direction, "rho_value": it.rho_value,
                              "members": [idx], "mask": member[idx].copy(), "last_idx": idx})
    if len(instances) > A.MAX_BC:
        raise UnsupportedComposition(f"{len(instances)} distinct rewrite boundaries "
                                     f"(at most {A.MAX_BC} in one fused plan)")
    inst_of_item = {}
    for n, ins_ in enumerate(instances):
        for idx in ins_["members"]:
            inst_of_item[idx] = n

    # per-node velocity planes (one velocity boundary per node)
    bc_vel = None
    vel_owner = np.full((nx, ny), -1, np.int32)
    for idx in rewrites:
        it = items[idx]
        if it.kind not in VELOCITY_KINDS or it.nodes.size == 0:
            continue
        if bc_vel is None:
            bc_vel = np.zeros((2, nx, ny), np.float32)
        nd = it.nodes
        v = it.velocity if it.velocity is not None else np.zeros((nd.shape[0], 2), np.float32)
        clash = vel_owner[nd[:, 0], nd[:, 1]] >= 0
        if clash.any():
            old = bc_vel[:, nd[clash, 0], nd[clash, 1]].T
            if not np.array_equal(old, v[clash]):
                raise UnsupportedComposition("a node has two velocity boundaries with different values")
        bc_vel[0, nd[:, 0], nd[:, 1]] = v[:, 0]
        bc_vel[1, nd[:, 0], nd[:, 1]] = v[:, 1]
        vel_owner[nd[:, 0], nd[:, 1]] = idx

    # programs: ordered instance list per node, as a base-(MAX_BC + 1) key
    # (a boundary merged into the previous instance adds nothing)
    seqs = {}
    node_prog = np.zeros((nx, ny), np.int64)
    if rewrites:
        base = A.MAX_BC + 1
        key = np.zeros(nx * ny, np.int64)
        length = np.zeros(nx * ny, np.int32)
        last = np.full(nx * ny, -1, np.int32)
        for idx in rewrites:
            n = inst_of_item.get(idx)
            nd = items[idx].nodes
            if n is None or nd.size == 0:
                continue
            lin = nd[:, 0].astype(np.int64) * ny + nd[:, 1]
            lin = lin[last[lin] != n]
            key[lin] = key[lin] * base + (n + 1)
            length[lin] += 1
            last[lin] = n
        if (length > A.PROG_LEN).any():
            q = int(np.flatnonzero(length > A.PROG_LEN)[0])
            raise UnsupportedComposition(f"node ({q // ny}, {q % ny}) has {int(length[q])} rewrite "
                                         f"boundaries (at most {A.PROG_LEN})")
        has = length > 0
        keys, inv = np.unique(key[has], return_inverse=True)
        if keys.size + 1 > A.MAX_PROG:
            raise UnsupportedComposition(f"{keys.size} distinct boundary programs "
                                         f"(at most {A.MAX_PROG - 1})")
        for pid, kv in enumerate(keys.tolist(), start=1):
            digits = []
            while kv:
                digits.append(kv % base - 1)
                kv //= base
            seqs[tuple(reversed(digits))] = pid
        flat = np.zeros(nx * ny, np.int64)
        flat[has] = inv + 1
        node_prog = flat.reshape(nx, ny)
    code |= node_prog << A.CODE_PROG_SHIFT
    code[save & active] |= A.CODE_SAVE

    programs = np.full((A.MAX_PROG, A.PROG_LEN), -1, np.int8)
    for t, pid in seqs.items():
        programs[pid, :len(t)] = t

    # --- segment flags: 0 when every node of the segment is plain
    seg_w = 32 * V
    nseg = (nx + seg_w - 1) // seg_w
    plain = code == A.CODE_ACTIVE  # (nx, ny)
    pad = nseg * seg_w - nx
    notplain = np.pad(~plain, ((0, pad), (0, 0)), constant_values=False)
    seg_flags = notplain.reshape(nseg, seg_w, ny).any(axis=1).T.astype(np.uint8)  # (ny, nseg)
    # lane masks: bit l of (y, seg) is set when one of lane l's V nodes is not plain
    lane_special = notplain.reshape(nseg, 32, V, ny).any(axis=2).transpose(2, 0, 1)  # (ny, nseg, 32)
    bits = (np.uint64(1) << np.arange(32, dtype=np.uint64))
    lane_mask = (lane_special.astype(np.uint64) * bits).sum(axis=2).astype(np.uint32)  # (ny, nseg)
    lanes = np.flatnonzero(lane_special.ravel()).astype(np.int32)  # (y * nseg + seg) * 32 + lane

    read_sites = None
    if in_place:
        _check_in_place(code, active)
        read_sites = _read_sites(items, rewrites, nx, ny)

    return CompiledPlan(code=code.astype(np.uint16), seg_flags=np.ascontiguousarray(seg_flags),
                        lane_mask=np.ascontiguousarray(lane_mask), lanes=lanes,
                        nseg=nseg, instances=instances, programs=programs, nprog=len(seqs) + 1,
                        bc_vel=bc_vel, items=items, active=active, save=save,
                        n_special_segments=int(seg_flags.sum()), read_sites=read_sites)


def _prev_rewrite(rewrites, idx):
    pos = rewrites.index(idx)
    return rewrites[pos - 1] if pos > 0 else None


OPP = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6])


def _check_in_place(code, active):
    """The in-place step pairs the locations a node reads and writes; that
    holds when every link cut by bounce-back is cut on both sides (node x
    bounces back link k from a colliding source x - c_k only if that source
    bounces back link opp(k) from x) and no colliding node streams from a
    node outside the collision group.  Sources wrap around the lattice, as
    the pull does."""
    for k in range(1, 9):
        shift = (int(CX[k]), int(CY[k]))
        src_active = np.roll(active, shift, axis=(0, 1))  # active[x - c_k]
        bounce = ((code >> (k - 1)) & 1).astype(bool)
        src_bounce_back = np.roll(((code >> (OPP[k] - 1)) & 1).astype(bool), shift, axis=(0, 1))
        one_sided = active & bounce & src_active & ~src_bounce_back
        if one_sided.any():
            i, j = np.argwhere(one_sided)[0]
            raise UnsupportedComposition(
                f"in-place step: node ({i}, {j}) bounces back link {k} from a colliding node that streams "
                "the opposite link from it (a link cut on one side only)")
        frozen = active & ~bounce & ~src_active
        if frozen.any():
            i, j = np.argwhere(frozen)[0]
            raise UnsupportedComposition(
                f"in-place step: node ({i}, {j}) streams link {k} from a node outside the collision group")


def _read_sites(items, rewrites, nx, ny):
    """(m, 2) int32 (x, y) of every node whose post-stream populations a
    boundary program reads (x - c_dir, and x - 2 c_dir for extrapolation),
    distinct and sorted by (y, x)."""
    pts = []
    for idx in rewrites:
        it = items[idx]
        if it.nodes.size == 0:
            continue
        _, _, x2_f, x3_f = READS[it.kind]
        d = np.array([CX[it.direction], CY[it.direction]], np.int32)
        if x2_f:
            pts.append(it.nodes - d)
        if x3_f:
            pts.append(it.nodes - 2 * d)
    if not pts:
        return np.zeros((0, 2), np.int32)
    q = np.unique(np.concatenate(pts).astype(np.int64) @ np.array([1, nx], np.int64))
    return np.stack([q % nx, q // nx], 1).astype(np.int32)
