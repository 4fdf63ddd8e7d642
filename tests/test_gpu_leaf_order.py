"""GPU parity of the kd leaf order on inputs chosen for each ordering path.

The leaf order of a candidate list (the order in which the reference's
kd-tree range query returns its points) is computed on the device by one of
three paths: the rank method (short lists), the sorted-axis split with lazy
qselect replay of tied nodes (lists up to 2048 entries, three size classes),
and the exact qselect replay (longer lists).  Each test builds inputs that
drive a path hard and requires the ordered hit list to equal the oracle's,
whose kd-tree follows the reference's qselect_r sequence literally.
"""

import numpy as np
import pytest

from test_gpu_parity import compare

pytestmark = pytest.mark.gpu


def _structures(seed, lengths, step=None):
    from pyjess_gb300 import workloads as W

    rngs = [np.random.default_rng([seed, i]) for i in range(len(lengths))]
    structs = W.make_structures(rngs, lengths, [1 + i % 3 for i in range(len(lengths))])
    if step:
        for s in structs:
            s["xyz"] = np.round(s["xyz"] / step) * step
    return structs


def _templates(seed, structs, n, **kw):
    from pyjess_gb300 import workloads as W

    rng = np.random.default_rng([seed, 99])
    return [W.make_template(rng, structs[int(rng.integers(len(structs)))], int(rng.integers(3, 6)), **kw)
            for _ in range(n)]


@pytest.mark.parametrize("mode", ["fp32", "fp64"])
def test_ties_on_a_coarse_grid(mode):
    """Coordinates on a 0.25 A grid: equal axis values on both sides of many
    median boundaries, so the sorted-axis path replays qselect on tied nodes
    and their ancestors."""
    from pyjess_gb300 import workloads as W

    structs = _structures(11, [120, 350, 800, 1300], step=0.25)
    specs = _templates(11, structs, 60)
    res, ref = compare(W.pack_templates(specs), W.pack(structs), mode=mode, rmsd_threshold=2.0,
                       distance_cutoff=1.5, max_dynamic_distance=1.5)
    st = res.stats()
    assert ref["hits"]["count"] > 0
    assert st["leaf_sorted"] > 0 and st["leaf_replays"] > 0


def test_every_size_class():
    """Backbone templates matching any residue: candidate lists of every
    structure's N / CA / C / O atoms, one structure per size class (up to 512,
    1024, 2048 entries, and beyond 2048 for the exact replay)."""
    from pyjess_gb300 import workloads as W

    structs = _structures(12, [400, 900, 1700, 2300], step=0.01)
    specs = _templates(12, structs, 4, permissive=True)
    res, ref = compare(W.pack_templates(specs), W.pack(structs), mode="fp32", rmsd_threshold=1.5,
                       distance_cutoff=1.0, max_dynamic_distance=1.0, max_candidates=40)
    st = res.stats()
    assert ref["hits"]["count"] > 0
    assert st["leaf_sorted"] > 0 and st["leaf_exact"] > 0


def test_non_finite_coordinate_is_rejected():
    """pjg_structures_create refuses a NaN or infinite coordinate with an
    invalid-argument error naming the structure and atom."""
    from pyjess_gb300 import _native
    from pyjess_gb300 import workloads as W

    for bad in (np.nan, np.inf):
        structs = _structures(13, [60, 60])
        structs[1]["xyz"] = structs[1]["xyz"].copy()
        structs[1]["xyz"][17, 0] = bad
        with pytest.raises(RuntimeError, match="structure 1 atom 17: non-finite coordinate"):
            _native.Structures(W.pack(structs))
