"""Protein Data Bank trajectories (nbody_simulation_result.jl:786-1001).

write_pdb_data writes one MODEL per saved time with the positions in
angstrom (x 10), wrapped into the cubic box; for water each molecule's H
sites keep their offsets from the wrapped O (whole molecules). The text
follows the reference's columns character for character: the same
`%8.3f` coordinates, paddings, record names and `REMARK 250 time=...` lines,
with Julia's printing of the time. extract_from_pdb reads the first two
MODELs of such a file back into water molecules as the reference does:
positions of the first model, velocities zero (the reference computes the
finite difference to the second model and then overwrites it with zero,
:988-994), masses 15.999 and 1.00794.

Host-side text I/O: the frames come from SimulationResult (solution frames
saved by the GPU step loop); nothing here runs on the GPU.
"""
import io as _io

import numpy as np

from .bodies import MassBody, WaterMolecule
from .parameters import _jl
from .systems import WaterSPCFw


def _hetatm_prefixes(names, residues, res_index, serials):
    """`HETATM` + lpad(serial, 5) + 2 spaces + rpad(name, 4) + residue +
    lpad(res_index, 6) + 4 spaces (write_pdb_data, :819-841 and :860-864)."""
    return ["HETATM" + str(s).rjust(5) + "  " + nm.ljust(4) + rs + str(ri).rjust(6) + "    "
            for s, nm, rs, ri in zip(serials, names, residues, res_index)]


def _line_formats(prefixes, elements):
    """Per atom, the format of its HETATM line: the prefix, three `%8.3f`
    coordinates (lpad 8 changes nothing: `%8.3f` is at least 8 wide),
    lpad("1.00", 6), lpad("0.00", 6), 10 spaces, lpad(element, 2), newline."""
    return [p + "%8.3f%8.3f%8.3f  1.00  0.00" + " " * 10 + el.rjust(2) + "\n" for p, el in zip(prefixes, elements)]


def _wrap(cc, L):
    """x - L floor(x / L), element by element (:800, :855)."""
    return cc - L * np.floor(cc / L)


def write_pdb_data(f, sr):
    """Write every saved time of a SimulationResult as a PDB MODEL
    (write_pdb_data, nbody_simulation_result.jl:792-876)."""
    sysm = sr.simulation.system
    from .simulation import get_position
    L = 10 * sr.simulation.boundary_conditions.L
    n = len(sysm.bodies)
    if isinstance(sysm, WaterSPCFw):
        mol = np.repeat(np.arange(1, n + 1), 3)
        prefixes = _hetatm_prefixes(["O", "H1", "H2"] * n, ["HOH"] * (3 * n), mol, range(1, 3 * n + 1))
        elements = ["O", "H", "H"] * n
        unit = "picoseconds"
    else:
        prefixes = _hetatm_prefixes(["Ar"] * n, ["Ar"] * n, range(1, n + 1), range(1, n + 1))
        elements = ["Ar"] * n
        unit = "steps"
    fmts = _line_formats(prefixes, elements)
    for count, t in enumerate(sr.solution.t, start=1):
        cc0 = 10 * get_position(sr, t)  # 3 x cols
        cc = _wrap(cc0, L)
        if isinstance(sysm, WaterSPCFw):
            # H sites: the wrapped O plus their unwrapped offsets, (cc_O + cc0_H) - cc0_O (:802-806)
            o = cc[:, 0::3]
            cc[:, 1::3] = (o + cc0[:, 1::3]) - cc0[:, 0::3]
            cc[:, 2::3] = (o + cc0[:, 2::3]) - cc0[:, 0::3]
        f.write("MODEL".ljust(10) + str(count) + "\n")
        f.write("REMARK 250 time=" + _jl(float(t)) + " " + unit + "\n")
        f.write("".join(map(str.__mod__, fmts, map(tuple, cc[:, : len(fmts)].T.tolist()))))
        f.write("ENDMDL\n")


def save_to_pdb(sr, path):
    """save_to_pdb(result, path) (:881-885)."""
    with open(path, "w") as f:
        write_pdb_data(f, sr)


def _sites(ln, f):
    """The O line and the next two (H1, H2) as three positions in nm: the
    6th-8th whitespace fields / 10 (:929-943)."""
    out = []
    for line in (ln, f.readline(), f.readline()):
        ps = line.split()
        out.append(np.array([float(ps[5]), float(ps[6]), float(ps[7])]) / 10)
    return out


def extract_from_pdb(f):
    """Water molecules from the first two MODELs of a PDB text stream
    (extract_from_pdb, nbody_simulation_result.jl:912-1001)."""
    if isinstance(f, str):
        f = _io.StringIO(f)
    cc = []
    wms = []

    def _skip_to_model():
        while True:
            ln = f.readline()
            if not ln or ln[:5] == "MODEL":
                return

    _skip_to_model()
    t1 = float(f.readline().split()[2][5:])
    while True:
        ln = f.readline()
        if not ln or ln[:6] == "ENDMDL":
            break
        if len(ln) > 13 and ln[13] == "O":
            cc.extend(_sites(ln, f))
    _skip_to_model()
    t2 = float(f.readline().split()[2][5:])
    _ = t2 - t1  # the reference's tau, used only by the velocities it then discards
    mc = 0
    while True:
        ln = f.readline()
        if not ln or ln[:6] == "ENDMDL":
            break
        if len(ln) > 13 and ln[13] == "O":
            mc += 1
            _sites(ln, f)
            o = MassBody(cc[3 * (mc - 1)], (0.0, 0.0, 0.0), 15.999)
            h1 = MassBody(cc[3 * (mc - 1) + 1], (0.0, 0.0, 0.0), 1.00794)
            h2 = MassBody(cc[3 * (mc - 1) + 2], (0.0, 0.0, 0.0), 1.00794)
            wms.append(WaterMolecule(o, h1, h2))
    return wms


def load_water_molecules_from_pdb(path):
    """load_water_molecules_from_pdb(path) (:906-910)."""
    with open(path) as f:
        return extract_from_pdb(f)
