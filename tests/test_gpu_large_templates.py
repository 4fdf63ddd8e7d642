"""Templates of more than 32 atoms against the oracle.

The reference takes templates of any size (Template.__init__,
src/pyjess/_jess.pyx:1825-1912).  libpjg searches templates of up to 32
atoms with k_search (one level per lane) and larger ones with
k_search_large; both run in the same query, so these workloads mix the two.
Templates of 11-14 residues x 3 atoms (33-42 atoms) are drawn from
synthetic donor structures within a 14 A sphere, next to ordinary 2-4
residue templates.  Bar as in test_gpu_parity.py: identical ordered hit
lists and search counters, RMSD within RMSD_TOL.
"""

import numpy as np
import pytest

from test_gpu_parity import compare

pytestmark = pytest.mark.gpu

PARAMS = dict(rmsd_threshold=2.0, distance_cutoff=1.5, max_dynamic_distance=1.5)


def mixed_workload(seed=4242, n_structures=12, n_templates=16):
    from pyjess_gb300 import workloads as W

    kids = np.random.SeedSequence(seed).spawn(n_structures + n_templates)
    meta = np.random.Generator(np.random.PCG64(kids[0]))
    lengths = meta.integers(200, 600, size=n_structures)
    chains = meta.integers(1, 4, size=n_structures)
    structs = W.make_structures([np.random.Generator(np.random.PCG64(k)) for k in kids[:n_structures]], lengths,
                                chains)
    specs = []
    for j in range(n_templates):
        rng = np.random.Generator(np.random.PCG64(kids[n_structures + j]))
        n_res = int(rng.integers(11, 15)) if j % 2 == 0 else int(rng.integers(2, 5))
        specs.append(W.make_template(rng, structs[j % n_structures], n_res, radius=14.0))
    pt, ps = W.pack_templates(specs), W.pack(structs)
    assert max(np.diff(pt.atom_offset)) > 32
    return pt, ps


@pytest.mark.parametrize("mode", ["fp32", "fp64", "plain"])
def test_large_templates_identical(mode):
    pt, ps = mixed_workload()
    res, ref = compare(pt, ps, mode=mode, **PARAMS)
    sizes = np.diff(ref["hits"]["atom_offset"])
    assert (sizes > 32).sum() > 0, "no hit of a template over 32 atoms"


@pytest.mark.parametrize("kw", [dict(best_match=True), dict(max_candidates=1), dict(max_candidates=3),
                                dict(best_match=True, max_candidates=2), dict(reorder=False),
                                dict(ignore_chain=1), dict(ignore_chain=2)])
def test_large_templates_query_options(kw):
    pt, ps = mixed_workload(seed=77)
    compare(pt, ps, mode="fp32", **PARAMS, **kw)
