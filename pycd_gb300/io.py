"""POSCAR input and plain-text run reports.

``read_poscar`` returns the same dictionary keys as PyCD/io.py:12-82
(``lattice_matrix``, ``element_types``, ``num_elements``, ``total_elements``,
``coordinate_type``, ``coordinates``, ``file_format``) so that ``Material``
builds the identical site order.  Like the reference, the universal scale
factor on line 2 is not applied.  ``generate_report`` writes the
``<name>.log`` files of PyCD/io.py:163-199 (prefix text, then the elapsed
time) so that downstream readers of those logs keep working.
"""
from datetime import datetime
from pathlib import Path

import numpy as np


def _floats(line, n=None):
    vals = [float(tok) for tok in line.split()]
    return vals if n is None else vals[:n]


def read_poscar(input_file_path):
    with open(input_file_path, "r") as fh:
        lines = fh.read().splitlines()
    # Element symbols either sit on line 6 (VASP 5) or on line 1 (VASP 4).
    line6 = lines[5].split()
    has_symbols = bool(line6) and line6[0].isalpha()
    lattice_matrix = np.array([_floats(lines[i], 3) for i in (2, 3, 4)],
                              dtype=np.float64)
    if has_symbols:
        element_types = line6
        counts_line, ctype_line, first = 6, 7, 8
    else:
        element_types = lines[0].split()
        counts_line, ctype_line, first = 5, 6, 7
    num_elements = np.array([int(tok) for tok in lines[counts_line].split()],
                            dtype=int)
    total_elements = int(num_elements.sum())
    coordinate_type = lines[ctype_line].split()[0]
    coordinates = np.zeros((total_elements, 3))
    for i in range(total_elements):
        coordinates[i, :] = _floats(lines[first + i], 3)
    width = len(lines[first].split()[0])
    file_format = {18: "VASP", 11: "VESTA"}.get(width, "unknown")
    return {
        "lattice_matrix": lattice_matrix,
        "element_types": element_types,
        "num_elements": num_elements,
        "total_elements": total_elements,
        "coordinate_type": coordinate_type,
        "coordinates": coordinates,
        "file_format": file_format,
    }


def write_poscar(dst_file_path, comment, lattice_matrix, element_types,
                 num_elements, fractional_coords):
    """Write a VASP-5 POSCAR with 'Direct' coordinates (synthetic lattices)."""
    out = [comment, "1.0"]
    for row in np.asarray(lattice_matrix, dtype=np.float64):
        out.append("  ".join(f"{v:20.10f}" for v in row))
    out.append("   ".join(element_types))
    out.append("   ".join(str(int(n)) for n in num_elements))
    out.append("Direct")
    for row in np.asarray(fractional_coords, dtype=np.float64):
        out.append("  ".join(f"{v:18.12f}" for v in row))
    Path(dst_file_path).write_text("\n".join(out) + "\n")


def generate_report(start_time, dst_path, file_name, print_time_elapsed,
                    prefix=None):
    report_file_path = Path(dst_path) / (file_name + ".log")
    elapsed = datetime.now() - start_time
    with open(report_file_path, "w") as report:
        if prefix:
            report.write(prefix)
        if print_time_elapsed:
            report.write(
                "Time elapsed: "
                + ("%2d days, " % elapsed.days if elapsed.days else "")
                + ("%2d hours" % ((elapsed.seconds // 3600) % 24))
                + (", %2d minutes" % ((elapsed.seconds // 60) % 60))
                + (", %2d seconds" % (elapsed.seconds % 60)))
    return None
