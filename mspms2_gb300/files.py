"""The reference's output files read and written on the host: the trajectory file
(trj.mspms, trajectory() of src/dumpxyz.c:37-66; written by the engine's integrators
through mg_traj_open) and the snapshot (ss.mspms, snapshot() of src/dumpxyz.c:19-35)."""
from __future__ import annotations

import numpy as np


def read_trajectory(path: str) -> dict:
    """Parses a trajectory file: {"nmole": [per species], "natom", "names": [per species
    list of names], "aw": [per species arrays], "frames": [n_frames, 3, natom]}."""
    b = open(path, "rb").read()
    o = 0

    def ints(k):
        nonlocal o
        v = np.frombuffer(b, np.int32, k, o)
        o += 4 * k
        return v

    nsp, nmole, natom = (int(v) for v in ints(3))
    names, aws, per = [], [], []
    for _ in range(nsp):
        nm, na = (int(v) for v in ints(2))
        per.append(nm)
        nl, al = [], []
        for _ in range(na):
            nl.append(b[o:o + 5].split(b"\0")[0].decode(errors="replace"))
            al.append(float(np.frombuffer(b, np.float64, 1, o + 5)[0]))
            o += 13
        names.append(nl)
        aws.append(np.array(al))
    frame = 4 * nsp + 24 * natom
    nf = (len(b) - o) // frame
    if o + nf * frame != len(b):
        raise ValueError(f"{path}: trailing bytes after {nf} frames")
    frames = np.empty((nf, 3, natom))
    for f in range(nf):
        q = o + f * frame
        if not np.array_equal(np.frombuffer(b, np.int32, nsp, q), per):
            raise ValueError(f"{path}: frame {f} molecule counts differ from the header")
        frames[f] = np.frombuffer(b, np.float64, 3 * natom, q + 4 * nsp).reshape(3, natom)
    return {"nmole": per, "natom": natom, "names": names, "aw": aws, "frames": frames, "total_mole": nmole}


def write_snapshot(path: str, system, istep: int, box, x, y, z) -> None:
    """The snapshot text file of snapshot() (src/dumpxyz.c:19-35): natom; istep and the box;
    one line per site with its template name and position (C's %lf: six decimals)."""
    names = [nm for sp in system.species for _ in range(sp.nmole) for nm in sp.atom_names]
    with open(path, "w") as f:
        f.write(f"{len(names)}\n")
        f.write(f"{istep} {box[0]:f} {box[1]:f} {box[2]:f}\n")
        for nm, a, b, c in zip(names, x, y, z):
            f.write(f"{nm}  {a:f}  {b:f}  {c:f}\n")
