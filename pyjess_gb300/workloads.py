"""Seeded synthetic workloads for the template-matching benchmarks.

No public dataset is available offline, so structures and templates are
generated with the shapes and value distributions of the benchmark
configurations (all randomness from ``numpy.random.PCG64``, base seed
20261203, per-configuration seed = base + index, per-item streams from
``SeedSequence.spawn``):

Structures
    C-alpha random walk with 3.8 A steps, bond angle U(90, 120) degrees,
    dihedral U(-180, 180) degrees; residue types i.i.d. from standard
    amino-acid background frequencies; the standard heavy atoms of each type
    (PDB names) placed around the C-alpha at ~1.5 A bond lengths;
    coordinates rounded to 0.001 A; serials 1..N; chains split contiguously.
Templates
    Residues within 10 A of a centre residue of a donor structure, 3 atoms
    per residue perturbed by N(0, 0.3 A); 1-3 residue names (the true one
    first), 1-2 atom names (the true one first); match mode drawn from the
    modes the reference fixtures pin (0, 1, 3); distance weight U(0, 1.5);
    chain and residue number copied from the donor.

Every function returns `PackedStructures` / `PackedTemplates`, the flat
arrays of the C ABI, so the benchmark never builds per-atom Python objects.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from ._pack import PackedStructures, PackedTemplates

BASE_SEED = 20261203

RESIDUES = {
    "ALA": ("N", "CA", "C", "O", "CB"),
    "ARG": ("N", "CA", "C", "O", "CB", "CG", "CD", "NE", "CZ", "NH1", "NH2"),
    "ASN": ("N", "CA", "C", "O", "CB", "CG", "OD1", "ND2"),
    "ASP": ("N", "CA", "C", "O", "CB", "CG", "OD1", "OD2"),
    "CYS": ("N", "CA", "C", "O", "CB", "SG"),
    "GLN": ("N", "CA", "C", "O", "CB", "CG", "CD", "OE1", "NE2"),
    "GLU": ("N", "CA", "C", "O", "CB", "CG", "CD", "OE1", "OE2"),
    "GLY": ("N", "CA", "C", "O"),
    "HIS": ("N", "CA", "C", "O", "CB", "CG", "ND1", "CD2", "CE1", "NE2"),
    "ILE": ("N", "CA", "C", "O", "CB", "CG1", "CG2", "CD1"),
    "LEU": ("N", "CA", "C", "O", "CB", "CG", "CD1", "CD2"),
    "LYS": ("N", "CA", "C", "O", "CB", "CG", "CD", "CE", "NZ"),
    "MET": ("N", "CA", "C", "O", "CB", "CG", "SD", "CE"),
    "PHE": ("N", "CA", "C", "O", "CB", "CG", "CD1", "CD2", "CE1", "CE2", "CZ"),
    "PRO": ("N", "CA", "C", "O", "CB", "CG", "CD"),
    "SER": ("N", "CA", "C", "O", "CB", "OG"),
    "THR": ("N", "CA", "C", "O", "CB", "OG1", "CG2"),
    "TRP": ("N", "CA", "C", "O", "CB", "CG", "CD1", "CD2", "NE1", "CE2", "CE3", "CZ2", "CZ3", "CH2"),
    "TYR": ("N", "CA", "C", "O", "CB", "CG", "CD1", "CD2", "CE1", "CE2", "CZ", "OH"),
    "VAL": ("N", "CA", "C", "O", "CB", "CG1", "CG2"),
}
RESNAMES = tuple(RESIDUES)
# background amino-acid frequencies (percent), in RESNAMES order
FREQ = np.array([8.25, 5.53, 4.06, 5.45, 1.37, 3.93, 6.75, 7.07, 2.27, 5.96,
                 9.66, 5.84, 2.42, 3.86, 4.70, 6.56, 5.34, 1.08, 2.92, 6.87])
FREQ = FREQ / FREQ.sum()


def _enc_name(name: str) -> bytes:
    b = name.encode()
    if len(b) < 4:
        b = b"_" + b
    return b.ljust(4, b"_")


_NAME_TABLE = {}
for _r, _names in RESIDUES.items():
    for _n in _names:
        _NAME_TABLE[_n] = np.frombuffer(_enc_name(_n), np.uint8)
_RES_TABLE = {r: np.frombuffer(r.encode() + b"\0", np.uint8) for r in RESIDUES}
_RES_ATOMS = [len(RESIDUES[r]) for r in RESNAMES]


def _seed(config: int, *extra) -> np.random.SeedSequence:
    return np.random.SeedSequence([BASE_SEED + config, *extra])


_MAXA = max(_RES_ATOMS)
_NAMES_BY_TYPE = np.zeros((len(RESNAMES), _MAXA, 4), np.uint8)
for _t, _r in enumerate(RESNAMES):
    for _j, _n in enumerate(RESIDUES[_r]):
        _NAMES_BY_TYPE[_t, _j] = _NAME_TABLE[_n]
_RES_BY_TYPE = np.stack([_RES_TABLE[r] for r in RESNAMES])
_COUNTS = np.asarray(_RES_ATOMS)


def _ca_traces(thetas, phis):
    """C-alpha random walks for several chains at once (natural extension
    reference frame placement): 3.8 A steps, bond angle theta, dihedral phi."""
    S = len(thetas)
    L = max(len(t) for t in thetas)
    th = np.zeros((S, L))
    ph = np.zeros((S, L))
    for i, (t, p) in enumerate(zip(thetas, phis)):
        th[i, :len(t)] = t
        ph[i, :len(p)] = p
    pos = np.zeros((S, L, 3))
    if L > 1:
        pos[:, 1, 0] = 3.8
    if L > 2:
        pos[:, 2] = pos[:, 1] + 3.8 * np.stack([-np.cos(th[:, 2]), np.sin(th[:, 2]), np.zeros(S)], 1)
    for i in range(3, L):
        a, b, c = pos[:, i - 3], pos[:, i - 2], pos[:, i - 1]
        bc = c - b
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        nrm = np.cross(b - a, bc)
        nn = np.linalg.norm(nrm, axis=1, keepdims=True)
        nrm = np.where(nn > 1e-9, nrm / np.maximum(nn, 1e-12), np.array([0.0, 0.0, 1.0]))
        m2 = np.cross(nrm, bc)
        d0 = -3.8 * np.cos(th[:, i])
        d1 = 3.8 * np.sin(th[:, i]) * np.cos(ph[:, i])
        d2 = 3.8 * np.sin(th[:, i]) * np.sin(ph[:, i])
        pos[:, i] = c + bc * d0[:, None] + m2 * d1[:, None] + nrm * d2[:, None]
    return [pos[i, :len(t)] for i, t in enumerate(thetas)]


def make_structures(rngs, lengths, chains, adversarial=False):
    """Synthetic proteins, one per generator in `rngs` (dicts of atom arrays)."""
    thetas, phis, draws = [], [], []
    for rng, n_res in zip(rngs, lengths):
        n_res = int(n_res)
        thetas.append(np.radians(rng.uniform(90, 120, size=n_res)))
        phis.append(np.radians(rng.uniform(-180, 180, size=n_res)))
        types = rng.choice(len(RESNAMES), size=n_res, p=FREQ)
        counts = _COUNTS[types]
        side = rng.normal(size=(n_res, 3))
        noise = rng.normal(size=(int(counts.sum()), 3))
        draws.append((types, counts, side, noise))
    cas = _ca_traces(thetas, phis)
    out = []
    for ca, (types, counts, side, noise), n_chains in zip(cas, draws, chains):
        n_res = len(ca)
        n = int(counts.sum())
        prev = np.empty_like(ca)
        nxt = np.empty_like(ca)
        if n_res > 1:
            prev[1:] = ca[:-1]
            prev[0] = ca[0] - (ca[1] - ca[0])
            nxt[:-1] = ca[1:]
            nxt[-1] = ca[-1] + (ca[-1] - ca[-2])
        else:
            prev[0] = ca[0] - np.array([3.8, 0, 0])
            nxt[0] = ca[0] + np.array([3.8, 0, 0])
        u = nxt - prev
        u /= np.linalg.norm(u, axis=1, keepdims=True) + 1e-12
        side = side - (side * u).sum(1, keepdims=True) * u
        side /= np.linalg.norm(side, axis=1, keepdims=True) + 1e-12
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
        res_of = np.repeat(np.arange(n_res), counts)
        j = np.arange(n) - starts[res_of]
        xyz = np.empty((n, 3))
        cr, ur, sr = ca[res_of], u[res_of], side[res_of]
        xyz[j == 1] = cr[j == 1]
        xyz[j == 0] = (cr - 1.46 * (0.8 * ur + 0.6 * sr))[j == 0]
        cpos = cr + 1.52 * (0.8 * ur - 0.6 * sr)
        xyz[j == 2] = cpos[j == 2]
        xyz[j == 3] = (cpos - 1.23 * sr)[j == 3]
        step = sr + 0.6 * noise
        step /= np.linalg.norm(step, axis=1, keepdims=True) + 1e-12
        step *= 1.5
        step[j < 4] = 0.0
        walk = np.cumsum(step, axis=0)
        base = walk[starts][res_of]  # cumulative sum before each residue's atom 0
        base = base - step[starts][res_of]
        sc = cr + (walk - base)
        xyz[j >= 4] = sc[j >= 4]
        bounds = np.linspace(0, n_res, int(n_chains) + 1).astype(int)
        chain_of_res = np.searchsorted(bounds[1:], np.arange(n_res), side="right")
        chain = np.empty((n, 2), np.uint8)
        chain[:, 0] = ord(" ")
        chain[:, 1] = ord("A") + chain_of_res[res_of]
        if not adversarial:
            xyz = np.round(xyz, 3)
        out.append({
            "xyz": xyz,
            "name": _NAMES_BY_TYPE[types[res_of], j],
            "resname": _RES_BY_TYPE[types[res_of]],
            "res_seq": (res_of + 1).astype(np.int32),
            "chain": chain,
            "serial": np.arange(1, n + 1, dtype=np.int32),
            "types": types,
            "counts": counts,
        })
    return out


def make_structure(rng: np.random.Generator, n_res: int, n_chains: int = 1, adversarial=False):
    """One synthetic protein: dict of per-atom arrays (not yet packed)."""
    return make_structures([rng], [n_res], [n_chains], adversarial)[0]


def pack(structs) -> PackedStructures:
    off = np.zeros(len(structs) + 1, np.int64)
    np.cumsum([len(s["xyz"]) for s in structs], out=off[1:])
    cat = lambda k: np.ascontiguousarray(np.concatenate([s[k] for s in structs]))
    return PackedStructures(atom_offset=off, xyz=cat("xyz"), name=cat("name"), resname=cat("resname"),
                            chain=cat("chain"), res_seq=cat("res_seq"), serial=cat("serial"))


@dataclass
class TemplateSpec:
    """Template atoms before packing."""
    code: list
    res_seq: list
    chain: list
    xyz: list
    weight: list
    names: list      # list of lists of 4-byte names
    resnames: list   # list of lists of 4-byte residue names


def make_template(rng: np.random.Generator, donor: dict, n_res: int, *, modes=(0, 1, 3),
                  mode_p=(0.4, 0.3, 0.3), permissive=False, radius=10.0, atoms_per_res=3):
    """Template from `n_res` residues of `donor` within `radius` of a centre residue."""
    starts = np.concatenate([[0], np.cumsum(donor["counts"])])
    nres = len(donor["counts"])
    ca = donor["xyz"][starts[:-1] + 1]
    centre = int(rng.integers(nres))
    d = np.linalg.norm(ca - ca[centre], axis=1)
    near = np.flatnonzero(d <= radius)
    near = near[near != centre]
    pick = [centre] + list(rng.choice(near, size=min(n_res - 1, len(near)), replace=False)) if len(near) else [centre]
    spec = TemplateSpec([], [], [], [], [], [], [])
    for r in pick:
        rname = RESNAMES[donor["types"][r]]
        names = RESIDUES[rname]
        m = len(names)
        if permissive:
            sel = [i for i, nm in enumerate(names) if nm in ("N", "CA", "C", "O")]
            sel = list(rng.choice(sel, size=min(atoms_per_res, len(sel)), replace=False))
        else:
            sel = list(rng.choice(m, size=min(atoms_per_res, m), replace=False))
        for j in sel:
            a = starts[r] + j
            pos = donor["xyz"][a] + rng.normal(scale=0.3, size=3)
            spec.xyz.append(pos)
            spec.res_seq.append(int(donor["res_seq"][a]))
            spec.chain.append(bytes(donor["chain"][a]))
            spec.weight.append(float(rng.uniform(0, 1.5)) if not permissive else 2.5)
            if permissive:
                spec.code.append(0)
                spec.resnames.append([_RES_TABLE[x].tobytes() for x in RESNAMES])
                spec.names.append([_enc_name(names[j])])
                continue
            mode = int(rng.choice(modes, p=mode_p))
            spec.code.append(mode)
            rn = [rname]
            extra = int(rng.integers(0, 3))
            others = [x for x in RESNAMES if x != rname]
            rn += list(rng.choice(others, size=extra, replace=False))
            spec.resnames.append([_RES_TABLE[x].tobytes() for x in rn])
            nm = [names[j]]
            if rng.random() < 0.5 and m > 1:
                alt = [x for x in names if x != names[j]]
                nm.append(str(rng.choice(alt)))
            spec.names.append([_enc_name(x) for x in nm])
    return spec


def pack_templates(specs) -> PackedTemplates:
    atom_offset = [0]
    code, res_seq, chain, xyz, weight = [], [], [], [], []
    name_off, names, rn_off, rns, dim = [0], [], [0], [], []
    for sp in specs:
        code += sp.code
        res_seq += sp.res_seq
        chain += sp.chain
        xyz += [tuple(p) for p in sp.xyz]
        weight += sp.weight
        for n_ in sp.names:
            names += n_
            name_off.append(len(names))
        for r_ in sp.resnames:
            rns += r_
            rn_off.append(len(rns))
        atom_offset.append(len(code))
        dim.append(len(set(zip(sp.res_seq, sp.chain))))
    return PackedTemplates(
        atom_offset=np.asarray(atom_offset, np.int32),
        code=np.asarray(code, np.int32),
        res_seq=np.asarray(res_seq, np.int32),
        chain=np.frombuffer(b"".join(chain), np.uint8).reshape(-1, 2).copy(),
        xyz=np.asarray(xyz, np.float64).reshape(-1, 3),
        dist_weight=np.asarray(weight, np.float64),
        name_offset=np.asarray(name_off, np.int32),
        names=np.frombuffer(b"".join(names), np.uint8).reshape(-1, 4).copy(),
        resname_offset=np.asarray(rn_off, np.int32),
        resnames=np.frombuffer(b"".join(rns), np.uint8).reshape(-1, 4).copy(),
        dim=np.asarray(dim, np.int32),
    )


def _zipf_residues(rng, n, lo=2, hi=8, a=2.0):
    k = np.arange(lo, hi + 1)
    p = k.astype(float) ** (-a)
    p /= p.sum()
    return rng.choice(k, size=n, p=p)


@dataclass
class Workload:
    name: str
    templates: PackedTemplates
    structures: PackedStructures
    params: dict
    notes: str = ""
    n_adversarial: int = 0      # structures 0 .. n_adversarial-1 are adversarial

    @property
    def pairs(self) -> int:
        return self.templates.n_templates * self.structures.n_structures


def config(index: int, *, scale: float = 1.0, n_structures=None, n_templates=None,
           residues=None, shard: int = 0) -> Workload:
    """Benchmark configuration `index` (0-4).  `scale` shrinks structure and
    template counts proportionally (parity tests run reduced instances);
    `residues` = (lo, hi) overrides the structure length range of config 4;
    `shard` > 0 draws an independent instance with the same distributions
    (one per rank of a multi-GPU run)."""
    ss = _seed(index) if shard == 0 else _seed(index, shard)
    if index == 0:
        rng = np.random.Generator(np.random.PCG64(ss))
        s = make_structure(rng, 300)
        spec = make_template(rng, s, 3)
        return Workload("cfg0: 1 structure (300 res) x 1 template (9 atoms)", pack_templates([spec]),
                        pack([s]), dict(rmsd_threshold=2.0, distance_cutoff=1.5, max_dynamic_distance=1.5))
    if index == 1:
        rng = np.random.Generator(np.random.PCG64(ss))
        s = make_structure(rng, 1000)
        nt = n_templates or max(1, int(round(200 * scale)))
        specs = [make_template(rng, s, int(rng.integers(3, 7))) for _ in range(nt)]
        return Workload(f"cfg1: 1 structure (1000 res) x {nt} templates (3-6 res)", pack_templates(specs),
                        pack([s]), dict(rmsd_threshold=2.0, distance_cutoff=1.5, max_dynamic_distance=1.5))
    if index in (2, 3):
        ns = n_structures or max(1, int(round((1000 if index == 2 else 2000) * scale)))
        nt = n_templates or max(1, int(round((2000 if index == 2 else 5000) * scale)))
        kids = ss.spawn(ns + nt + 1)
        meta = np.random.Generator(np.random.PCG64(kids[-1]))
        lengths = np.clip(np.round(np.exp(np.log(350) + 0.6 * meta.normal(size=ns))), 80, 3000).astype(int)
        chains = meta.integers(1, 5, size=ns)
        n_adv = 200 if index == 3 and ns >= 200 else (int(round(ns * 0.1)) if index == 3 else 0)
        structs = make_structures([np.random.Generator(np.random.PCG64(kids[i])) for i in range(ns)],
                                  lengths, chains)
        res_counts = _zipf_residues(meta, nt)
        donors = meta.integers(0, ns, size=nt)
        specs = []
        for j in range(nt):
            rng = np.random.Generator(np.random.PCG64(kids[ns + j]))
            specs.append(make_template(rng, structs[donors[j]], int(res_counts[j])))
        params = dict(rmsd_threshold=2.0, distance_cutoff=1.5, max_dynamic_distance=1.5)
        notes = ""
        if n_adv:
            _make_adversarial(structs, specs, donors, list(range(n_adv)), params, meta)
            notes = f"{n_adv} adversarial structures"
        label = "cfg2" if index == 2 else "cfg3"
        return Workload(f"{label}: {ns} structures x {nt} templates", pack_templates(specs), pack(structs),
                        params, notes, n_adv)
    if index == 4:
        ns = n_structures or max(1, int(round(500 * scale)))
        nt = n_templates or max(1, int(round(500 * scale)))
        kids = ss.spawn(ns + nt + 1)
        meta = np.random.Generator(np.random.PCG64(kids[-1]))
        lo, hi = residues if residues else (2000, 5000)
        lengths = meta.integers(lo, hi + 1, size=ns)
        structs = make_structures([np.random.Generator(np.random.PCG64(kids[i])) for i in range(ns)],
                                  lengths, meta.integers(1, 5, size=ns))
        donors = meta.integers(0, ns, size=nt)
        specs = [make_template(np.random.Generator(np.random.PCG64(kids[ns + j])), structs[donors[j]],
                               int(meta.integers(2, 4)), permissive=True, atoms_per_res=2)
                 for j in range(nt)]
        return Workload(f"cfg4: {ns} structures x {nt} permissive templates", pack_templates(specs),
                        pack(structs), dict(rmsd_threshold=3.0, distance_cutoff=3.0, max_dynamic_distance=3.0,
                                            max_candidates=10000))
    raise ValueError(index)


def _make_adversarial(structs, specs, donors, which, params, rng):
    """Move atoms of the `which` structures so that about 10% of the template
    pair distances of templates drawn from them sit within 1e-6 A of the
    annulus boundary d_jk +- theta_jk (coordinates keep full precision)."""
    r, s = params["distance_cutoff"], params["max_dynamic_distance"]
    which = set(which)
    for j, sp in enumerate(specs):
        if donors[j] not in which:
            continue
        st = structs[donors[j]]
        n = len(sp.code)
        for a in range(n):
            for b in range(a + 1, n):
                if rng.random() >= 0.10:
                    continue
                # molecule atoms with the template atoms' residue and name
                ia = _find_atom(st, sp, a)
                ib = _find_atom(st, sp, b)
                if ia is None or ib is None:
                    continue
                d = float(np.sqrt(((np.asarray(sp.xyz[a]) - np.asarray(sp.xyz[b])) ** 2).sum()))
                theta = min(r + sp.weight[a] + sp.weight[b], s)
                target = d + theta if rng.random() < 0.5 else max(d - theta, 0.5)
                target += float(rng.uniform(-1e-6, 1e-6))
                v = st["xyz"][ib] - st["xyz"][ia]
                nv = np.linalg.norm(v)
                if nv < 1e-9 or target <= 0:
                    continue
                st["xyz"][ib] = st["xyz"][ia] + v * (target / nv)


def _find_atom(st, sp, k):
    want_res = sp.res_seq[k]
    want_name = sp.names[k][0]
    idx = np.flatnonzero(st["res_seq"] == want_res)
    for i in idx:
        if st["name"][i].tobytes() == want_name and bytes(st["chain"][i]) == sp.chain[k]:
            return int(i)
    return None
