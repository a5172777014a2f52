"""VTK output of DG functions on the structured grid.

The counterpart of dune-fem's VTKIO / SubsamplingVTKIO (io/file/vtkio.hh),
which hand a discrete function to dune-grid's (subsampling) VTK writer: here
the grid is a Cartesian box, so the output is one VTK XML ImageData file
(.vti) with cell data.  Each grid cell is split into 2**level sub-cells per
direction and the DG function (tensor orthonormal Legendre basis, dof layout
cell * n^3 + i0 n^2 + i1 n + i2 with i0 the x-degree) is evaluated at the
sub-cell centres; level 0 writes the value at the cell centre.

This is output, not part of the compute path: the coefficients are read back
from the device once and evaluated with numpy.
"""
import base64
import os

import numpy as np


def legendre_table(order, points):
    """L_i(x) = sqrt(2i+1) P_i(2x-1) on [0,1] at the points: array [len(points), order+1]."""
    x = 2.0 * np.asarray(points, dtype=np.float64) - 1.0
    out = np.empty((x.size, order + 1))
    for i in range(order + 1):
        c = np.zeros(i + 1)
        c[i] = 1.0
        out[:, i] = np.sqrt(2 * i + 1) * np.polynomial.legendre.legval(x, c)
    return out


def evaluate_subcells(coeffs, cells, order, level=0):
    """Values of the DG function at the sub-cell centres: array [Nz*S, Ny*S, Nx*S], S = 2**level."""
    nx, ny, nz = cells
    n = order + 1
    S = 2 ** level
    u = np.asarray(coeffs, dtype=np.float64).reshape(nz, ny, nx, n, n, n)  # [..., i0 (x), i1 (y), i2 (z)]
    L = legendre_table(order, (np.arange(S) + 0.5) / S)  # [S, n]
    v = np.einsum("zyxabc,pa,qb,rc->zryqxp", u, L, L, L, optimize=True)
    return v.reshape(nz * S, ny * S, nx * S)


def _b64(arr):
    raw = np.ascontiguousarray(arr).tobytes()
    return base64.b64encode(np.uint64(len(raw)).tobytes() + raw).decode("ascii")


def write_vti(path, cells, order, fields, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0), level=0):
    """Writes fields {name: dof vector (numpy array or DeviceArray)} of DG Q_order
    functions on the cells grid to path (.vti appended if missing).  Returns the path."""
    if not path.endswith(".vti"):
        path += ".vti"
    nx, ny, nz = cells
    S = 2 ** level
    ext = (nx * S, ny * S, nz * S)
    spacing = [(upper[k] - lower[k]) / ext[k] for k in range(3)]
    parts = []
    for name, vec in fields.items():
        arr = vec.numpy() if hasattr(vec, "numpy") and not isinstance(vec, np.ndarray) else np.asarray(vec)
        vals = evaluate_subcells(arr.astype(np.float64), cells, order, level)
        parts.append('      <DataArray type="Float64" Name="%s" format="binary">\n%s\n      </DataArray>\n'
                     % (name, _b64(vals.ravel())))
    whole = "0 %d 0 %d 0 %d" % ext
    text = ('<?xml version="1.0"?>\n'
            '<VTKFile type="ImageData" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
            '  <ImageData WholeExtent="%s" Origin="%r %r %r" Spacing="%r %r %r">\n'
            '    <Piece Extent="%s">\n'
            '      <CellData>\n%s      </CellData>\n'
            '    </Piece>\n'
            '  </ImageData>\n'
            '</VTKFile>\n') % (whole, lower[0], lower[1], lower[2], spacing[0], spacing[1], spacing[2], whole,
                               "".join(parts))
    d = os.path.dirname(os.path.abspath(path))
    os.makedirs(d, exist_ok=True)
    with open(path, "w") as f:
        f.write(text)
    return path


def read_vti_cell_data(path):
    """Reads back the cell data of a file written by write_vti: {name: array [Nz*S, Ny*S, Nx*S]}."""
    import xml.etree.ElementTree as ET
    root = ET.parse(path).getroot()
    img = root.find("ImageData")
    x0, x1, y0, y1, z0, z1 = (int(t) for t in img.get("WholeExtent").split())
    out = {}
    for da in img.find("Piece").find("CellData"):
        blob = base64.b64decode(da.text.strip())
        nbytes = int(np.frombuffer(blob[:8], dtype=np.uint64)[0])
        out[da.get("Name")] = np.frombuffer(blob[8:8 + nbytes], dtype=np.float64).reshape(z1 - z0, y1 - y0, x1 - x0)
    return out


class VTKIO:
    """Writes numbered snapshots name-000000.vti, ... (DataOutput / VTKIO usage
    in a time loop, io/file/dataoutput.hh, io/file/vtkio.hh)."""

    def __init__(self, prefix, cells, order, lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0), level=0):
        self.prefix, self.cells, self.order = prefix, cells, order
        self.lower, self.upper, self.level = lower, upper, level
        self.count = 0

    def write(self, fields):
        path = write_vti("%s-%06d.vti" % (self.prefix, self.count), self.cells, self.order, fields,
                         self.lower, self.upper, self.level)
        self.count += 1
        return path
