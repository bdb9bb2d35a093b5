"""Seeded molecular test systems for the bond-constraint path: rigid dimers,
linear trimers, triangles and free atoms on a lattice of molecule centres.
Synthetic (the reference ships no molecular input files)."""
import numpy as np


def _unit(rng, n):
    u = rng.normal(size=(n, 3))
    return u / np.linalg.norm(u, axis=1, keepdims=True)


def molecular_mix(cells, spacing, seed, bond=1.0, kinds=("dimer", "trimer", "triangle", "free")):
    """Molecules on a simple cubic lattice of centres `spacing` apart, kind
    cycling through `kinds`. Returns r (n,3), box (3,), bbi, bbj, length (per
    constraint, 0-based) and the molecule id of every atom."""
    rng = np.random.default_rng(seed)
    g = np.arange(cells)
    centres = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) * spacing
    box = np.full(3, cells * spacing)
    centres = centres - box / 2.0 + spacing / 2.0
    r, bbi, bbj, ln, mol = [], [], [], [], []
    for m, c in enumerate(centres):
        kind = kinds[m % len(kinds)]
        u = _unit(rng, 1)[0]
        base = len(r)
        if kind == "dimer":
            r += [c + 0.5 * bond * u, c - 0.5 * bond * u]
            bbi.append(base); bbj.append(base + 1); ln.append(bond)
        elif kind == "trimer":
            # bent chain A-B-C, two constraints sharing B
            w = _unit(rng, 1)[0]
            w = w - (w @ u) * u
            w /= np.linalg.norm(w)
            b = c
            a = b + bond * u
            cc = b + bond * (np.cos(2.0) * u + np.sin(2.0) * w)
            r += [a, b, cc]
            bbi += [base, base + 1]; bbj += [base + 1, base + 2]; ln += [bond, bond]
        elif kind == "triangle":
            w = _unit(rng, 1)[0]
            w = w - (w @ u) * u
            w /= np.linalg.norm(w)
            p0 = c
            p1 = c + bond * u
            p2 = c + bond * (0.5 * u + np.sqrt(0.75) * w)
            r += [p0, p1, p2]
            bbi += [base, base + 1, base + 2]; bbj += [base + 1, base + 2, base]; ln += [bond] * 3
        else:
            r.append(c)
        mol += [m] * (len(r) - base)
    return (np.array(r), box, np.array(bbi, dtype=np.int32), np.array(bbj, dtype=np.int32), np.array(ln),
            np.array(mol))


def polymer_chains(counts, length, seed, bond=1.0, spacing=1.6, jitter=0.05):
    """Planar zig-zag chains (bond angle 120 degrees, all-trans) of `length`
    beads running along x, on a counts[1] x counts[2] grid in (y, z) and
    counts[0] chains end to end along x, with seeded jitter. Returns r (n,3),
    box (3,), bonds (nb,2), bends (na,3), dihedrals (nd,4), all 0-based."""
    rng = np.random.default_rng(seed)
    step_x = bond * np.cos(np.radians(30.0))
    chain_x = length * step_x + spacing
    box = np.array([counts[0] * chain_x, counts[1] * spacing, counts[2] * spacing])
    r, bonds, bends, dihs = [], [], [], []
    for a in range(counts[0]):
        for b in range(counts[1]):
            for c in range(counts[2]):
                base = len(r)
                for k in range(length):
                    r.append([a * chain_x + k * step_x, b * spacing + (k % 2) * 0.5 * bond, c * spacing])
                bonds += [[base + k, base + k + 1] for k in range(length - 1)]
                bends += [[base + k, base + k + 1, base + k + 2] for k in range(length - 2)]
                dihs += [[base + k, base + k + 1, base + k + 2, base + k + 3] for k in range(length - 3)]
    r = np.array(r) - box / 2.0 + 0.25
    r += jitter * np.clip(rng.normal(size=r.shape), -3, 3)
    return (r, box, np.array(bonds, dtype=np.int32), np.array(bends, dtype=np.int32),
            np.array(dihs, dtype=np.int32))
