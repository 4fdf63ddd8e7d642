"""Shared helpers of the test-suite (result conversion, comparisons)."""

import numpy as np


class ArraysResult:
    """Adapter so `_materialize` can build Hit objects from oracle arrays."""

    def __init__(self, hits):
        self._hits = hits

    def arrays(self):
        return self._hits


def oracle_hits(jess, molecules, **kwargs):
    from oracle import oracle
    from pyjess_gb300._jess import _materialize
    from pyjess_gb300._pack import pack_molecules

    r = oracle.query(jess._packed_templates(), pack_molecules(molecules), **kwargs)
    return _materialize(ArraysResult(r["hits"]), jess, molecules), r


def hit_keys(h):
    """(structure, template, ordinal, atoms...) tuples of a hit array dict."""
    out = []
    for i in range(h["count"]):
        a0, a1 = int(h["atom_offset"][i]), int(h["atom_offset"][i + 1])
        out.append((int(h["structure"][i]), int(h["template"][i]), int(h["ordinal"][i]),
                    tuple(int(x) for x in h["atoms"][a0:a1])))
    return out


def parse_block(block):
    lines = block.strip().splitlines()
    query_id, rmsd, template_id, _, det, _, loge = lines[0].split()
    return query_id, float(rmsd), float(det), float(loge), lines[1:-1]
