"""The likelihood map build (createTSDFMap, map_util.h:17-154) pinned to the oracle
and to the reference's own CudaSubVoxelMap ctor + setData (CPU).

The product builds 16-bit slot codes (tsdfl_build_map_codes) whose values come
from a 601-entry table (tsdfl_code_values).  Both are compared here with
independent computations: the table entry by entry with the oracle's
restatement of map_util.h:68-71,124-127, and whole maps -- coefficients, brick
table, every slot's value bit for bit and the free-space cells -- with the
oracle's createTSDFMap restatement and, where the reference's sources were
compiled on this machine, with the reference's own map built from the same
tuples.  The worlds are the bench's and the batch's: a room at 0.064 m (the
reference's 64-cell chunks) and at 0.05 m, a 25 x 25 m part of the
100x100x10 m building at 0.05 m in 8^3 chunks, a warehouse and a tunnel at
0.1 m in 16^3 chunks.
"""
import numpy as np
import pytest

from oracle import oracle_py as O
from tsdf_localization_gb300 import build_map_codes, code_values, synth

COEF_FIELDS = [f for f, _ in O.Coef._fields_]


def _named_order(pos, raw):
    """Chunks in the order createTSDFMap visits them: the group's member names
    "<x>_<y>_<z>" in byte order."""
    names = ["%d_%d_%d" % tuple(p) for p in pos]
    order = sorted(range(len(names)), key=lambda i: names[i].encode())
    return np.ascontiguousarray(pos[order]), np.ascontiguousarray(raw[order])


def _coef_tuple(c):
    return tuple(getattr(c, f) for f in COEF_FIELDS)


@pytest.mark.parametrize("sigma", [0.1, 0.05, 0.2])
def test_code_values_equal_oracle_likelihood(sigma):
    """All 600 |tsdf| codes and the init value, bit for bit."""
    init = O.likelihood_init(sigma)
    vals = code_values(sigma, init)
    want = np.array([O.likelihood_value(v, sigma) for v in range(600)] + [init], np.float32)
    assert vals.dtype == np.float32 and vals.shape == (601,)
    assert np.array_equal(vals.view(np.uint32), want.view(np.uint32))
    # map_util.h:68-71 underflows to 0 at sigma 0.1; the largest value is at |tsdf| = 0
    assert vals[0] == vals.max()


# (name, world, seed, voxel mm, chunk edge, chunks kept along x and y from the
# low corner or None for all): the building is checked on a 25 x 25 m part of
# its chunks (every floor, the same cells and chunking), which runs in a tenth
# of the whole building's time.
WORLDS = [
    ("room@0.064/64", synth.ROOM, 4, 64, 64, None),
    ("room@0.05/8", synth.ROOM, 21, 50, 8, None),
    ("building@0.05/8 25x25m", synth.BUILDING, 2, 50, 8, 62),
    ("warehouse@0.1/16", synth.WAREHOUSE, 23, 100, 16, None),
    ("tunnel@0.1/16", synth.TUNNEL, 24, 100, 16, None),
]


@pytest.mark.parametrize("name,kind,seed,voxel_mm,edge,crop", WORLDS, ids=[w[0] for w in WORLDS])
def test_map_build_equals_oracle_and_reference(name, kind, seed, voxel_mm, edge, crop):
    pos, raw = synth.World(kind, seed).tsdf_chunks(voxel_mm, edge)
    if crop is not None:
        keep = (pos[:, 0] < pos[:, 0].min() + crop) & (pos[:, 1] < pos[:, 1].min() + crop)
        pos, raw = pos[keep], raw[keep]
    pos, raw = _named_order(pos, raw)
    coef, grid_occ, codes, free_xyz = build_map_codes(pos, raw, edge, voxel_mm, 0.1, want_free=True)
    om, ofree = O.OracleMap.from_chunks(pos, raw, voxel_mm, 0.1, edge=edge)
    assert _coef_tuple(coef) == _coef_tuple(om.coef)
    assert np.array_equal(grid_occ, om.grid_occ)
    vals = np.append(code_values(0.1, coef.init_value), np.float32(coef.init_value))
    assert codes.max() <= 600
    got = vals[codes]
    assert got.shape == om.data.shape
    assert np.array_equal(got.view(np.uint32), om.data.view(np.uint32))
    assert np.array_equal(free_xyz, ofree)
    del om
    if not O.reference_available():
        pytest.skip("the reference's sources are not compiled on this machine")
    t = O.chunk_tuples(pos, raw, voxel_mm, 0.1, edge=edge)
    del raw
    rm = O.RefMap(t["min"], t["max"], np.float32(voxel_mm * 0.001), t["init"], t["tuples"])
    assert _coef_tuple(rm.coef) == _coef_tuple(coef)
    assert np.array_equal(rm.grid_occ(), grid_occ)
    assert np.array_equal(rm.data().view(np.uint32), got.view(np.uint32))
