"""Seeded synthetic workloads with the shapes and value distributions of the
benchmark configurations (no public dataset is involved; PDB input is user data).

Bodies use the reference layout (resaxslib/include/utils.hpp:61-88): an
``(N, 4) float32`` array whose column 3 holds the uint32 type index bit for bit.

Generators
----------
* ``random_walk_chain``: 3-D random walk with fixed step length, each new atom
  rejected (and re-drawn) if it comes within ``self_avoid`` of an earlier atom.
* ``confined_chain``: random walk with fixed step length whose steps are
  re-drawn while they would leave a sphere of radius ``R``; used for the compact
  chains (R = Rg * sqrt(5/3), the radius of a uniform ball with that Rg) and for
  the chain "folded into a 60 A sphere".
* ``exp_form_factors``: one-body factors f_t(q) = Z_t * exp(-b_t q^2).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "pack_bodies", "body_types", "random_walk_chain", "confined_chain", "draw_types",
    "exp_form_factors", "q_grid", "Workload", "make_config", "CONFIG_NAMES",
]


def pack_bodies(xyz: np.ndarray, types: np.ndarray) -> np.ndarray:
    """(N,3) positions + (N,) uint types -> (N,4) float32 bodies, type bits in .w."""
    xyz = np.asarray(xyz, dtype=np.float32)
    out = np.empty((len(xyz), 4), np.float32)
    out[:, :3] = xyz
    out.view(np.uint32)[:, 3] = np.asarray(types, dtype=np.uint32)
    return out


def body_types(bodies: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(bodies, dtype=np.float32).view(np.uint32)[:, 3].copy()


def _unit_vectors(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def random_walk_chain(n: int, rng: np.random.Generator, step: float = 3.8,
                      self_avoid: float = 3.0, max_tries: int = 200) -> np.ndarray:
    """Self-avoiding random walk: a step is re-drawn while the new atom lies
    closer than ``self_avoid`` to any earlier atom (after ``max_tries`` failed
    draws the last draw is kept, which never happened for the sizes used here)."""
    pos = np.zeros((n, 3), np.float64)
    cell = self_avoid
    grid: dict[tuple[int, int, int], list[int]] = {}

    def key(p):
        return (int(math.floor(p[0] / cell)), int(math.floor(p[1] / cell)),
                int(math.floor(p[2] / cell)))

    def clash(p):
        k = key(p)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                        d = p - pos[j]
                        if d @ d < self_avoid * self_avoid:
                            return True
        return False

    grid.setdefault(key(pos[0]), []).append(0)
    pool = _unit_vectors(rng, 4 * n + 64)
    pi = 0
    for i in range(1, n):
        for _ in range(max_tries):
            if pi >= len(pool):
                pool = _unit_vectors(rng, 4 * n + 64)
                pi = 0
            cand = pos[i - 1] + step * pool[pi]
            pi += 1
            if not clash(cand):
                break
        pos[i] = cand
        grid.setdefault(key(cand), []).append(i)
    return pos


def confined_chain(n: int, rng: np.random.Generator, radius: float, step: float = 3.8,
                   max_tries: int = 100) -> np.ndarray:
    """Random walk of fixed step length confined to a ball of ``radius``."""
    pos = np.zeros((n, 3), np.float64)
    pool = _unit_vectors(rng, 2 * n + 64)
    pi = 0
    r2 = radius * radius
    for i in range(1, n):
        prev = pos[i - 1]
        for _ in range(max_tries):
            if pi >= len(pool):
                pool = _unit_vectors(rng, 2 * n + 64)
                pi = 0
            cand = prev + step * pool[pi]
            pi += 1
            if cand @ cand <= r2:
                break
        else:  # step toward the centre
            cand = prev - step * prev / max(np.linalg.norm(prev), 1e-9)
        pos[i] = cand
    return pos


def draw_types(n: int, rng: np.random.Generator, probs) -> np.ndarray:
    probs = np.asarray(probs, np.float64)
    return rng.choice(len(probs), size=n, p=probs / probs.sum()).astype(np.uint32)


def q_grid(n_q: int, q_max: float, q_min: float = 0.0) -> np.ndarray:
    return np.linspace(q_min, q_max, n_q).astype(np.float32)


def exp_form_factors(q: np.ndarray, Z, b) -> np.ndarray:
    """[n_q][T] float32 table f_t(q) = Z_t exp(-b_t q^2)."""
    q = np.asarray(q, np.float64)[:, None]
    return (np.asarray(Z, np.float64)[None, :] * np.exp(-np.asarray(b, np.float64)[None, :] * q * q)
            ).astype(np.float32)


@dataclass
class Workload:
    name: str
    q: np.ndarray                 # (n_q,) float32
    ff: np.ndarray                # (n_q, T) float32
    bodies: np.ndarray            # (N, 4) float32
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.bodies)

    @property
    def pairs(self) -> int:
        return self.n * (self.n - 1) // 2

    @property
    def pair_q(self) -> int:
        return self.pairs * len(self.q)


TYPE_P5 = (0.6, 0.15, 0.15, 0.05, 0.05)
Z5 = (6, 7, 8, 16, 1)
Z8 = (1, 6, 7, 8, 15, 16, 26, 30)

CONFIG_NAMES = {
    1: "plain_forward_n2000_q101",
    2: "recalc_sasa_n20000_q201",
    3: "adjoint_n50000_q256",
    4: "precision_n200000_q512",
    5: "batch_256_members_q201",
}


def make_config(idx: int, seed: int = 0, n_override: int | None = None) -> Workload:
    """Synthetic workload for benchmark configuration ``idx`` (1..4).

    ``n_override`` shrinks the atom count while keeping every other parameter
    (used by parity tests that must finish in seconds on the CPU oracle)."""
    rng = np.random.default_rng(1000 + 17 * idx + seed)
    if idx == 1:
        n = n_override or 2000
        xyz = random_walk_chain(n, rng)
        types = draw_types(n, rng, TYPE_P5)
        q = q_grid(101, 0.5)
        ff = exp_form_factors(q, Z5, rng.uniform(0.5, 2.0, 5))
    elif idx == 2:
        n = n_override or 20000
        rg = 25.0 * (n / 20000) ** (1 / 3)
        xyz = confined_chain(n, rng, rg * math.sqrt(5 / 3))
        types = draw_types(n, rng, TYPE_P5)
        q = q_grid(201, 0.5)
        ff = exp_form_factors(q, Z5, rng.uniform(0.5, 2.0, 5))
    elif idx == 3:
        n = n_override or 50000
        rg = 25.0 * (n / 20000) ** (1 / 3)
        xyz = confined_chain(n, rng, rg * math.sqrt(5 / 3))
        types = draw_types(n, rng, TYPE_P5)
        q = q_grid(256, 0.6)
        ff = exp_form_factors(q, Z5, rng.uniform(0.5, 2.0, 5))
    elif idx == 4:
        n = n_override or 200000
        radius = 60.0 * (n / 200000) ** (1 / 3)
        xyz = confined_chain(n, rng, radius)
        types = draw_types(n, rng, (1,) * 8)
        q = q_grid(512, 1.0)
        ff = exp_form_factors(q, Z8, rng.uniform(0.3, 2.5, 8))
    else:
        raise ValueError(f"no single-structure config {idx}")
    return Workload(CONFIG_NAMES[idx], q, ff, pack_bodies(xyz, types))


def batch_members(n_members: int = 256, seed: int = 0, n_lo: int = 1000, n_hi: int = 30000,
                  scale: float = 1.0):
    """Config 5: independent seeded chains with N ~ U[n_lo, n_hi] (optionally
    scaled down for tests).  Returns (q, ff, list of bodies arrays)."""
    rng = np.random.default_rng(5000 + seed)
    q = q_grid(201, 0.5)
    ff = exp_form_factors(q, Z5, rng.uniform(0.5, 2.0, 5))
    sizes = rng.integers(n_lo, n_hi + 1, size=n_members)
    sizes = np.maximum(2, (sizes * scale).astype(int))
    members = []
    for m, n in enumerate(sizes):
        r = np.random.default_rng(rng.integers(1 << 62))
        rg = 25.0 * (n / 20000) ** (1 / 3)
        xyz = confined_chain(int(n), r, rg * math.sqrt(5 / 3))
        members.append(pack_bodies(xyz, draw_types(int(n), r, TYPE_P5)))
    return q, ff, members


# ----------------------------------------------------------------------------
# synthetic PDB files (input of the calc_saxs CLI)
# ----------------------------------------------------------------------------

# heavy atoms of the 20 standard residues (PDB atom names)
RESIDUE_ATOMS = {
    "ALA": ["CB"], "ARG": ["CB", "CG", "CD", "NE", "CZ", "NH1", "NH2"],
    "ASN": ["CB", "CG", "OD1", "ND2"], "ASP": ["CB", "CG", "OD1", "OD2"],
    "CYS": ["CB", "SG"], "GLN": ["CB", "CG", "CD", "OE1", "NE2"],
    "GLU": ["CB", "CG", "CD", "OE1", "OE2"], "GLY": [],
    "HIS": ["CB", "CG", "ND1", "CD2", "CE1", "NE2"], "ILE": ["CB", "CG1", "CG2", "CD1"],
    "LEU": ["CB", "CG", "CD1", "CD2"], "LYS": ["CB", "CG", "CD", "CE", "NZ"],
    "MET": ["CB", "CG", "SD", "CE"],
    "PHE": ["CB", "CG", "CD1", "CD2", "CE1", "CE2", "CZ"], "PRO": ["CB", "CG", "CD"],
    "SER": ["CB", "OG"], "THR": ["CB", "OG1", "CG2"],
    "TRP": ["CB", "CG", "CD1", "CD2", "NE1", "CE2", "CE3", "CZ2", "CZ3", "CH2"],
    "TYR": ["CB", "CG", "CD1", "CD2", "CE1", "CE2", "CZ", "OH"],
    "VAL": ["CB", "CG1", "CG2"],
}


def _pdb_atom_line(rec, serial, name, alt, res, chain, resseq, xyz, element, short=False):
    # PDB columns: name in 13-16 (1-letter elements start in column 14)
    nm = (" " + name) if len(name) < 4 and len(element.strip()) <= 1 else name
    line = (f"{rec:<6}{serial % 100000:>5} {nm:<4}{alt}{res:>3} {chain}{resseq % 10000:>4}    "
            f"{xyz[0]:8.3f}{xyz[1]:8.3f}{xyz[2]:8.3f}{1.0:6.2f}{20.0:6.2f}")
    if short:
        return line
    return line + " " * 10 + f"{element:>2}  "


def write_synthetic_pdb(path: str, n_residues: int = 60, n_models: int = 2, seed: int = 0,
                        quirks: bool = True) -> None:
    """Writes a protein-like PDB file: a random-walk backbone of standard
    residues with their heavy atoms (and some hydrogens) placed around each
    residue, one MODEL per conformation.  With ``quirks`` it also holds the
    records and fields the reader must skip or map: waters, alternate
    locations, hydrogens, a HETATM zinc, an unknown element, a blank element
    field, lines without element columns and an over-long line."""
    rng = np.random.default_rng(seed)
    names = sorted(RESIDUE_ATOMS)
    seq = [names[i] for i in rng.integers(0, len(names), n_residues)]
    base = random_walk_chain(n_residues, rng, step=3.8)
    lines = ["HEADER    SYNTHETIC TEST STRUCTURE", "REMARK   1 GENERATED"]
    for m in range(n_models):
        ca = base + rng.normal(0.0, 0.4 * m, base.shape)
        lines.append(f"MODEL     {m + 1:>4}")
        serial = 1
        for r, res in enumerate(seq):
            atoms = ["N", "CA", "C", "O"] + RESIDUE_ATOMS[res]
            for a in atoms:
                xyz = ca[r] + rng.normal(0.0, 1.2, 3)
                el = "S" if a[0] == "S" else a[0]
                short = quirks and rng.random() < 0.05
                if quirks and rng.random() < 0.05:
                    el = " "  # blank element field
                lines.append(_pdb_atom_line("ATOM", serial, a, " ", res, "A", r + 1, xyz, el,
                                            short=short))
                serial += 1
            if quirks and r % 7 == 3:  # alternate locations: A kept, B dropped
                xyz = ca[r] + rng.normal(0.0, 1.2, 3)
                lines.append(_pdb_atom_line("ATOM", serial, "CB", "A", res, "A", r + 1, xyz, "C"))
                lines.append(_pdb_atom_line("ATOM", serial + 1, "CB", "B", res, "A", r + 1,
                                            xyz + 0.3, "C"))
                serial += 2
            if quirks and r % 5 == 1:  # hydrogens are skipped
                lines.append(_pdb_atom_line("ATOM", serial, "HA", " ", res, "A", r + 1,
                                            ca[r] + 1.0, "H"))
                serial += 1
        if quirks:
            lines.append("TER")
            lines.append(_pdb_atom_line("HETATM", serial, "ZN", " ", " ZN", "A", 900,
                                        ca[0] + 2.0, "Zn"))
            lines.append(_pdb_atom_line("HETATM", serial + 1, "FE", " ", "HEM", "A", 901,
                                        ca[1] + 2.0, "Fe"))
            lines.append(_pdb_atom_line("HETATM", serial + 2, "O", " ", "HOH", "A", 950,
                                        ca[2] + 3.0, "O"))
            long = _pdb_atom_line("ATOM", serial + 3, "CA", " ", "GLY", "B", 999, ca[3] + 2.5, "C")
            lines.append(long + " " * 30 + "TRAILING-COLUMNS-BEYOND-99")
        lines.append("ENDMDL")
    lines.append("END" + " " * 77)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
