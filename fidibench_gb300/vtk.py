"""ASCII VTK writer for the upwind field.

Writes the same RECTILINEAR_GRID layout as the reference's C++ writer
(upwind/cxx/saveVTK.h:1-60): axis order reversed for VTK (the last array axis
varies fastest), node coordinates 0 + dx*i, CELL_DATA scalars ``f`` printed
with C++ stream default formatting (6 significant digits, %g), ten values per
line.  The file format has to match for the files to diff against the
reference's up0.vtk / up1.vtk; the code is written from the format, not
copied.
"""
from __future__ import annotations

import numpy as np


def _g(x: float) -> str:
    return "%g" % x


def write_rectilinear(fname: str, num_cells, deltas, f, title: str = "upwind.cxx") -> None:
    n = [int(x) for x in num_cells]
    nd = len(n)
    f = np.asarray(f, dtype=np.float64).reshape(-1)
    lines = ["# vtk DataFile Version 2.0\n", f"{title}\n", "ASCII\n",
             "DATASET RECTILINEAR_GRID\n"]
    dims = "DIMENSIONS"
    dims += f" {n[2] + 1}" if nd > 2 else " 1"
    dims += f" {n[1] + 1}" if nd > 1 else " 1"
    dims += f" {n[0] + 1}"
    lines.append(dims)

    def axis(label: str, k: int | None) -> str:
        if k is None:
            return f"\n{label} 1 double\n0.0\n"
        pts = "".join(" " + _g(0.0 + deltas[k] * i) for i in range(n[k] + 1))
        return f"\n{label} {n[k] + 1} double\n{pts}"

    lines.append(axis("X_COORDINATES", 2 if nd > 2 else None))
    lines.append(axis("Y_COORDINATES", 1 if nd > 1 else None))
    lines.append(axis("Z_COORDINATES", 0))
    lines.append(f"\nCELL_DATA {f.size}\nSCALARS f double 1\nLOOKUP_TABLE default\n")
    body = []
    for i, x in enumerate(f):
        body.append(_g(x) + " ")
        if (i + 1) % 10 == 0:
            body.append("\n")
    lines.append("".join(body))
    lines.append("\n")
    with open(fname, "w") as fh:
        fh.write("".join(lines))


def write_structured_filter(fname: str, global_dims, xmins, xmaxs, field, name: str) -> None:
    """The Filter's VTK file (cxx/writeVTK.cpp:11-95): STRUCTURED_GRID with
    node points in column-major order (x fastest) computed as
    lo + (hi - lo) * i / n, axes beyond the field's given extent 1 on [0, 1],
    then one cell value per line; floats printed with C++ stream defaults."""
    nd = len(global_dims)
    if nd > 3:
        return  # the reference warns and writes nothing for more than 3 axes
    lo, hi, cells = [0.0] * 3, [1.0] * 3, [1] * 3
    for d in range(nd):
        lo[d], hi[d], cells[d] = float(xmins[d]), float(xmaxs[d]), int(global_dims[d])
    nodes = [c + 1 for c in cells]
    f = np.asarray(field, dtype=np.float64).reshape(-1)
    out = ["# vtk DataFile Version 2.0\n", "produced by laplacian\n", "ASCII\n",
           "DATASET STRUCTURED_GRID\n", f"DIMENSIONS {nodes[0]} {nodes[1]} {nodes[2]}\n",
           f"POINTS {nodes[0] * nodes[1] * nodes[2]} float\n"]
    coords = [[lo[d] + (hi[d] - lo[d]) * i / float(cells[d]) for i in range(nodes[d])]
              for d in range(3)]
    for k in range(nodes[2]):
        for j in range(nodes[1]):
            for i in range(nodes[0]):
                out.append(f"{_g(coords[0][i])} {_g(coords[1][j])} {_g(coords[2][k])}\n")
    out.append(f"CELL_DATA {cells[0] * cells[1] * cells[2]}\n")
    out.append(f"SCALARS {name} float\n")
    out.append("LOOKUP_TABLE default\n")
    out.extend(_g(x) + "\n" for x in f)
    with open(fname, "w") as fh:
        fh.write("".join(out))
