"""Reader of the legacy VTK dumps the C++ driver writes (io.cpp): returns
(header line, points (nnd,2), cells (nel,4) 0-based, {name: cell array},
{name: point array})."""
import numpy as np


def read_vtk(path):
    with open(path) as f:
        lines = f.read().split("\n")
    assert lines[0].startswith("# vtk DataFile") and lines[2] == "ASCII"
    title = lines[1]
    i = 4
    pts = cells = None
    cell_data, point_data = {}, {}
    section = None
    while i < len(lines):
        w = lines[i].split()
        if not w:
            i += 1
            continue
        if w[0] == "POINTS":
            n = int(w[1])
            pts = np.array([[float(t) for t in lines[i + 1 + k].split()[:2]] for k in range(n)])
            i += 1 + n
        elif w[0] == "CELLS":
            n = int(w[1])
            cells = np.array([[int(t) for t in lines[i + 1 + k].split()[1:]] for k in range(n)])
            i += 1 + n
        elif w[0] == "CELL_TYPES":
            n = int(w[1])
            assert all(lines[i + 1 + k] == "9" for k in range(n))
            i += 1 + n
        elif w[0] in ("CELL_DATA", "POINT_DATA"):
            section = (cell_data if w[0] == "CELL_DATA" else point_data, int(w[1]))
            i += 1
        elif w[0] == "SCALARS":
            store, n = section
            conv = int if w[2] == "int" else float
            store[w[1]] = np.array([conv(lines[i + 2 + k]) for k in range(n)])
            i += 2 + n
        elif w[0] == "VECTORS":
            store, n = section
            store[w[1]] = np.array([[float(t) for t in lines[i + 1 + k].split()[:2]]
                                    for k in range(n)])
            i += 1 + n
        else:
            raise ValueError("unexpected line %r" % lines[i])
    return title, pts, cells, cell_data, point_data
