"""Seeded synthetic VSVB inputs in VALENCE's input format (README.md:146-246,
xm_module.F90:25-335), for the benchmark workloads:

  water_vshf   O + 2 H (0.96 A, 104.5 deg), 5 DOCC, 13 Cartesian functions
               (O: 3s 2p, H: 2s, 3 primitives per shell), FP64 energy.
  ch_chain     8-atom linear C/H chain (1.1 A), 4 Rumer-coupled pairs
               (16 determinants per side) + 8 DOCC, s/p/d basis of 104
               functions (C: 3s 2p 1d, H: 2s 1p 1d, 3-6 primitives).
  lif_cluster  4x4x4 cluster of Z=3/Z=9 at 2.0 A, s/p basis (3s 2p per
               atom, 576 functions), 304 DOCC on 1-2 atoms.
  batch        independent molecules of 2-12 atoms, Z in {1,3,6,7,8,9},
               s/p/d, 0-2 coupled pairs, DOCC for the rest.

Exponents are log-uniform, contraction coefficients uniform(0.1, 1) (the
code renormalises them, valence.F90:2264-2305), orbital weights
uniform(-1, 1) over the functions of each orbital's atoms (normalised
internally, valence.F90:2157-2182).  numpy.random.default_rng(seed).
"""
import math

import numpy as np


def _shells(rng, spec, lo, hi, nprim):
    out = []
    for l in spec:
        n = int(rng.integers(nprim[0], nprim[1] + 1))
        e = np.sort(np.exp(rng.uniform(math.log(lo), math.log(hi), n)))[::-1]
        c = rng.uniform(0.1, 1.0, n)
        out.append((l, list(zip(e, c))))
    return out


def _nfun(shells):
    return sum((l + 1) * (l + 2) // 2 for l, _ in shells)


def write_input(path, atoms, types, orbitals, npair=0, nunpd=0, pairs=None, ntol=(20, 16, 16)):
    """atoms: [(type, x, y, z)] in Angstrom; types: [(Z, shells)];
    orbitals: [(atom list (1-based), weights over the OBS functions)] in the
    order coupled, unpaired, DOCC."""
    ndocc = len(orbitals) - 2 * npair - nunpd
    totlen = sum(len(w) for _, w in orbitals)
    xpmax = max(len(w) for _, w in orbitals)
    num_sh = sum(len(s) for _, s in types)
    num_pr = sum(len(p) for _, s in types for _, p in s)
    nang = max(l for _, s in types for l, _ in s)
    mxctr = max(len(a) for a, _ in orbitals)
    nspinc = 1 if npair > 0 else 0
    L = [f"{len(atoms)} {len(types)} {npair} {nunpd} {ndocc} {totlen} {xpmax} {nspinc} {num_sh} {num_pr} {nang} 0 0 0 {mxctr}",
         f"{ntol[0]} {ntol[1]} {ntol[2]} 6 6 0 0.0 0.0"]
    for t, x, y, z in atoms:
        L.append(f"{t} {x:.10f} {y:.10f} {z:.10f}")
    for zc, shells in types:
        L.append(f"{zc:.1f} {len(shells)}")
        for l, prims in shells:
            L.append(f"{l} {len(prims)}")
            for e, c in prims:
                L.append(f"{e:.10e}" if len(prims) == 1 else f"{e:.10e} {c:.10f}")
    if npair > 0:
        L.append(" ".join(f"{a} {b}" for a, b in pairs))
    for atl, w in orbitals:
        L.append(f"{len(atl)} " + " ".join(str(a) for a in atl) + f" {len(w)}")
        L.append(" ".join(f"{k + 1} {v:.12f}" for k, v in enumerate(w)))
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def water_vshf(path, seed=1):
    rng = np.random.default_rng(seed)
    o = _shells(rng, [0, 0, 0, 1, 1], 0.1, 5000.0, (3, 3))
    h = _shells(rng, [0, 0], 0.1, 20.0, (3, 3))
    th = math.radians(104.5) / 2
    r = 0.96
    atoms = [(1, 0.0, 0.0, 0.0), (2, 0.0, r * math.sin(th), r * math.cos(th)), (2, 0.0, -r * math.sin(th), r * math.cos(th))]
    nf = {1: _nfun(o), 2: _nfun(h)}
    obs = [[1], [1], [1, 2], [1, 3], [1]]
    orbs = [(a, rng.uniform(-1, 1, sum(nf[atoms[i - 1][0]] for i in a))) for a in obs]
    write_input(path, atoms, [(8.0, o), (1.0, h)], orbs)
    return path


def ch_chain(path, seed=2, natom=8, npair=4, ndocc=8):
    rng = np.random.default_rng(seed)
    c = _shells(rng, [0, 0, 0, 1, 1, 2], 0.08, 3000.0, (3, 6))
    h = _shells(rng, [0, 0, 1, 2], 0.08, 3000.0, (3, 6))
    atoms = [((1 if i % 2 == 0 else 2), 0.0, 0.0, 1.1 * i) for i in range(natom)]
    nf = {1: _nfun(c), 2: _nfun(h)}
    norb = 2 * npair + ndocc
    orbs = []
    for i in range(norb):
        a = i % (natom - 1)
        atl = [a + 1, a + 2]
        orbs.append((atl, rng.uniform(-1, 1, sum(nf[atoms[k - 1][0]] for k in atl))))
    pairs = [(2 * k + 1, 2 * k + 2) for k in range(npair)]
    write_input(path, atoms, [(6.0, c), (1.0, h)], orbs, npair=npair, pairs=pairs)
    return path


def lif_cluster(path, seed=3, n=4, ndocc=304, spacing=2.0):
    rng = np.random.default_rng(seed)
    li = _shells(rng, [0, 0, 0, 1, 1], 0.05, 1e4, (3, 6))
    f = _shells(rng, [0, 0, 0, 1, 1], 0.05, 1e4, (3, 6))
    atoms = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                atoms.append((1 if (i + j + k) % 2 == 0 else 2, spacing * i, spacing * j, spacing * k))
    nf = {1: _nfun(li), 2: _nfun(f)}
    nat = len(atoms)
    orbs = []
    for o in range(ndocc):
        a = o % nat
        if o // nat % 2 == 0:
            atl = [a + 1]
        else:
            b = (a + 1) % nat
            atl = [a + 1, b + 1]
        orbs.append((atl, rng.uniform(-1, 1, sum(nf[atoms[k - 1][0]] for k in atl))))
    write_input(path, atoms, [(3.0, li), (9.0, f)], orbs, ntol=(20, 16, 12))
    return path


_ZB = {1: [0, 0, 1], 3: [0, 0, 0, 1], 6: [0, 0, 0, 1, 1, 2], 7: [0, 0, 0, 1, 1, 2], 8: [0, 0, 0, 1, 1, 2],
       9: [0, 0, 0, 1, 1, 2]}


def random_molecule(path, seed, nat_range=(2, 12), zs=(1, 3, 6, 7, 8, 9), min_sep=0.9, nfun_max=80):
    rng = np.random.default_rng(seed)
    while True:
        nat = int(rng.integers(nat_range[0], nat_range[1] + 1))
        z = [int(rng.choice(zs)) for _ in range(nat)]
        xyz = []
        while len(xyz) < nat:
            p = rng.uniform(-1.8, 1.8, 3) * (nat ** (1 / 3))
            if all(np.linalg.norm(p - q) >= min_sep for q in xyz):
                xyz.append(p)
        tz = sorted(set(z))
        types = [(float(zz), _shells(rng, _ZB[zz], 0.1, 2000.0, (3, 4))) for zz in tz]
        nf = {i + 1: _nfun(s) for i, (_, s) in enumerate(types)}
        atoms = [(tz.index(zz) + 1, *p) for zz, p in zip(z, xyz)]
        if sum(nf[a[0]] for a in atoms) <= nfun_max:
            break
    nelec = sum(z)
    npair = int(rng.integers(0, 3))
    npair = min(npair, nelec // 2)
    rest = nelec - 2 * npair
    nunpd = rest % 2
    ndocc = rest // 2
    norb = 2 * npair + nunpd + ndocc
    orbs = []
    for o in range(norb):
        a = int(rng.integers(0, nat))
        atl = [a + 1] if (o % 2 == 0 or nat == 1) else [a + 1, (a + 1) % nat + 1]
        orbs.append((atl, rng.uniform(-1, 1, sum(nf[atoms[k - 1][0]] for k in atl))))
    pairs = [(2 * k + 1, 2 * k + 2) for k in range(npair)]
    write_input(path, atoms, types, orbs, npair=npair, nunpd=nunpd, pairs=pairs)
    return path


def batch_molecules(dirpath, n=256, seed0=1000):
    """n independent random molecules (2-12 atoms, Z in {1,3,6,7,8,9}, 4-80
    functions, 0-2 coupled pairs, DOCC for the rest, one unpaired orbital when
    the electron count is odd), seeds seed0, seed0+1, ...  Returns the paths."""
    import os
    return [random_molecule(os.path.join(dirpath, f"mol{seed0 + i:05d}.inp"), seed0 + i) for i in range(n)]


def lif_cluster_small(path, seed=3):
    """The cluster workload's geometry and basis family at 2x2x2 (8 atoms, 72
    functions, 12 DOCC): a size the CPU oracle evaluates in seconds."""
    return lif_cluster(path, seed=seed, n=2, ndocc=12)


def alkane_chain(path, seed=4, ncarbon=42, nh=86, npair=8, ndocc=117):
    """The large optimisation loop's geometry: a zigzag chain of ncarbon Z=6
    atoms at 1.54 A with nh Z=1 atoms at 1.09 A (two per carbon, one more on
    each end carbon), s/p/d basis (C: 3s 2p 1d, H: 2s 1p 1d; 3-6 primitives,
    exponents log-uniform in [0.08, 3000]), npair Rumer pairs on
    neighbouring carbons and ndocc doubly occupied orbitals on 1-2 atoms.
    Defined for completeness: its size (about 1,500 functions, 65,536
    determinant pairs) is beyond what the GPU path runs."""
    rng = np.random.default_rng(seed)
    c = _shells(rng, [0, 0, 0, 1, 1, 2], 0.08, 3000.0, (3, 6))
    h = _shells(rng, [0, 0, 1, 2], 0.08, 3000.0, (3, 6))
    th = math.radians(109.5) / 2
    atoms = []
    for i in range(ncarbon):
        atoms.append((1, 1.54 * math.sin(th) * i, 0.0, (0.0 if i % 2 == 0 else 1.54 * math.cos(th))))
    hpos = []
    for i in range(ncarbon):
        x, y, z = atoms[i][1:]
        zd = -1.0 if i % 2 == 0 else 1.0
        for sgn in (1, -1):
            hpos.append((x, sgn * 1.09 * math.sin(th), z + zd * 1.09 * math.cos(th)))
    hpos.append((atoms[0][1] - 1.09, 0.0, atoms[0][3]))
    hpos.append((atoms[-1][1] + 1.09, 0.0, atoms[-1][3]))
    atoms += [(2, *p) for p in hpos[:nh]]
    nf = {1: _nfun(c), 2: _nfun(h)}
    orbs = []
    for k in range(2 * npair + ndocc):
        a = k % (ncarbon - 1)
        atl = [a + 1, a + 2] if k < 2 * npair or k % 2 == 0 else [a + 1]
        orbs.append((atl, rng.uniform(-1, 1, sum(nf[atoms[j - 1][0]] for j in atl))))
    pairs = [(2 * k + 1, 2 * k + 2) for k in range(npair)]
    write_input(path, atoms, [(6.0, c), (1.0, h)], orbs, npair=npair, pairs=pairs)
    return path


def lif_cluster_3(path, seed=3):
    """The cluster workload at 3x3x3 (27 atoms, 243 functions, 108 DOCC): the
    block-mode kernels at the full cluster's chunk size, small enough for a
    detailed profile."""
    return lif_cluster(path, seed=seed, n=3, ndocc=108)


def singular_pair_large(path, seed=5, natom=32, ndocc=32):
    """A spin-coupled pair whose first orbital sits on an atom 25 A away from
    a chain of natom Z=1 atoms (s, s, p shells, 5 functions each) that
    carries the second orbital and ndocc doubly occupied orbitals on 1-2
    atoms: every transition determinant pair that moves the far orbital into
    the other spin block has an exactly singular overlap block (a row of
    zeros up to exp(-300)), here with ndocc + 1 = 33 electrons of one spin."""
    rng = np.random.default_rng(seed)
    hsh = _shells(rng, [0, 0, 1], 0.3, 30.0, (3, 3))
    atoms = [(1, 0.0, 0.0, 1.4 * i) for i in range(natom)] + [(1, 25.0, 0.0, 0.0)]
    nf = _nfun(hsh)
    far = natom + 1
    orbs = [([far], rng.uniform(-1, 1, nf)), ([1, 2], rng.uniform(-1, 1, 2 * nf))]
    for k in range(ndocc):
        a = k % natom
        atl = [a + 1] if k < natom else [a + 1, (a + 1) % natom + 1]
        orbs.append((atl, rng.uniform(-1, 1, nf * len(atl))))
    write_input(path, atoms, [(1.0, hsh)], orbs, npair=1, pairs=[(1, 2)])
    return path


def describe(path):
    """Counts of an input in VALENCE's format (line A of xm_input and the
    basis records): atoms, shells, Cartesian functions, highest angular
    momentum, orbitals by kind, spin couplings, determinant pairs and
    weights -- the configuration fields of a benchmark line."""
    toks = open(path).read().split()
    it = iter(toks)
    a = [int(next(it)) for _ in range(15)]
    natom, natom_t, npair, nunpd, ndocc, totlen, _, nspinc = a[:8]
    for _ in range(8):
        next(it)
    types = []
    for _ in range(natom):
        types.append(int(next(it)))
        for _ in range(3):
            next(it)
    nfun_t, nsh_t, lmax = [], [], 0
    for _ in range(natom_t):
        next(it)
        ns = int(next(it))
        nf = 0
        for _ in range(ns):
            l, npr = int(next(it)), int(next(it))
            lmax = max(lmax, l)
            nf += (l + 1) * (l + 2) // 2
            for _ in range(npr if npr == 1 else 2 * npr):
                next(it)
        nfun_t.append(nf)
        nsh_t.append(ns)
    nsc = max(nspinc, 1)
    return {"atoms": natom, "shells": sum(nsh_t[t - 1] for t in types),
            "functions": sum(nfun_t[t - 1] for t in types), "max_l": lmax, "coupled_pairs": npair,
            "unpaired": nunpd, "docc": ndocc, "spatial_orbitals": 2 * npair + nunpd + ndocc,
            "spin_couplings": nsc, "determinant_pairs": nsc * nsc * 4 ** npair, "weights": totlen}


WORKLOADS = {"water_vshf": water_vshf, "ch_chain": ch_chain, "lif_cluster": lif_cluster,
             "lif_cluster_small": lif_cluster_small, "lif_cluster_3": lif_cluster_3, "alkane_chain": alkane_chain,
             "singular_pair_large": singular_pair_large}
