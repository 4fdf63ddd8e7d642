"""pjg_superpose_noalloc: the allocation-free superposition entry point.

Callers that cannot allocate device memory while they run (a real-time
loop, an application whose memory manager owns every device allocation) pass
their own input and output buffers; the entry point's only scratch is a
static device array inside the library.  This test
calls it through the C ABI on the hits of a normal `pjg_query` and checks that
it reproduces that query's rmsd, rotations and centroids, twice in a row
(the second call reuses the static scratch left by the first).  The file is
named so that pytest collects it last.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RMSD_TOL = 1e-9
ROT_TOL = 1e-7


def _bind():
    from pyjess_gb300 import _native

    L = _native.init()
    f = L.pjg_superpose_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.pjg_noalloc_last_error.restype = C.c_char_p
    return L


def test_superpose_noalloc_matches_query(golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from pyjess_gb300 import Jess, Molecule, Template, _native
    from pyjess_gb300._abi import QueryParams
    from pyjess_gb300._pack import pack_molecules

    L = _bind()
    amy = Molecule.load(str(golden / "1AMY.pdb"))
    t133 = Template.load(str(golden / "1.3.3.tpl"))
    t412 = Template.load(str(golden / "4.1.2.tpl"))
    jess = Jess([t133, t412])
    pt = jess._packed_templates()
    ps = pack_molecules([amy])
    P = QueryParams(rmsd_threshold=2.0, distance_cutoff=4.0, max_dynamic_distance=4.0, max_candidates=-1,
                    ignore_chain=0, best_match=0, reorder=1, mode=_native.MODE_BATCHED_FP32)
    ref = _native.query(_native.Templates(pt), _native.Structures(ps), P).arrays()
    assert ref["count"] > 100

    dev = torch.device("cuda")
    for t in range(pt.n_templates):
        rows = np.flatnonzero(ref["template"] == t)
        if len(rows) == 0:
            continue
        n = int(pt.atom_offset[t + 1] - pt.atom_offset[t])
        atoms = np.stack([ref["atoms"][ref["atom_offset"][i]:ref["atom_offset"][i + 1]] for i in rows])
        mol = torch.tensor(ps.xyz[atoms].reshape(-1), dtype=torch.float64, device=dev)
        tpl = torch.tensor(pt.xyz[pt.atom_offset[t]:pt.atom_offset[t + 1]].reshape(-1), dtype=torch.float64,
                           device=dev)
        m = len(rows)
        rmsd = torch.empty(m, dtype=torch.float64, device=dev)
        rot = torch.empty(9 * m, dtype=torch.float64, device=dev)
        cen = torch.empty(6 * m, dtype=torch.float64, device=dev)
        pass_rows = torch.empty(m, dtype=torch.int32, device=dev)
        pass_count = torch.empty(1, dtype=torch.int32, device=dev)
        # second call: a threshold between the hits' rmsds, so the ordered
        # compaction keeps a strict subset
        thresholds = (2.0, float(np.median(ref["rmsd"][rows])))
        for threshold in thresholds:
            torch.cuda.synchronize()
            st = L.pjg_superpose_noalloc(mol.data_ptr(), tpl.data_ptr(), m, n, threshold, rmsd.data_ptr(),
                                         rot.data_ptr(), cen.data_ptr(), pass_rows.data_ptr(),
                                         pass_count.data_ptr(), None)
            assert st == 0, L.pjg_noalloc_last_error()
            torch.cuda.synchronize()
            r = rmsd.cpu().numpy()
            assert np.abs(r - ref["rmsd"][rows]).max() <= RMSD_TOL
            assert np.abs(rot.cpu().numpy().reshape(m, 9) - ref["rotation"][rows]).max() <= ROT_TOL
            assert np.abs(cen.cpu().numpy().reshape(m, 6) - ref["centres"][rows]).max() <= 1e-9
            expect = np.flatnonzero(ref["rmsd"][rows] <= threshold)
            k = int(pass_count.cpu().item())
            assert k == len(expect)
            assert np.array_equal(pass_rows.cpu().numpy()[:k], expect)


def test_superpose_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    L = _bind()
    count = torch.empty(1, dtype=torch.int32, device="cuda")
    st = L.pjg_superpose_noalloc(None, None, (1 << 20) + 1, 9, 2.0, None, None, None, None, count.data_ptr(), None)
    assert st == 1
    assert b"at most" in L.pjg_noalloc_last_error()
