"""VTK XML rectilinear-grid writer (.vtr), standing in for pyevtk's
``gridToVTK`` used by the reference's ``export_VTK``
(Single_phase/LBM_3D_SinglePhase_Solver.py:462-475).  Point data are written
x-fastest (VTK order) as raw appended binary, one UInt64 byte count per block.
"""
import numpy as np

_VTK_TYPES = {
    np.dtype(np.int8): "Int8", np.dtype(np.uint8): "UInt8", np.dtype(np.int32): "Int32",
    np.dtype(np.int64): "Int64", np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64",
}


def grid_to_vtk(path, x, y, z, point_data):
    """Write ``path + '.vtr'``.  point_data: name -> (nx,ny,nz) array, or a
    3-tuple of such arrays for a vector field.  Returns the file name."""
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    nx, ny, nz = len(x), len(y), len(z)
    blocks = []
    arrays_xml = []
    offset = 0

    def add_block(raw):
        nonlocal offset
        blocks.append(np.uint64(len(raw)).tobytes() + raw)
        off = offset
        offset += 8 + len(raw)
        return off

    for name, val in point_data.items():
        if isinstance(val, (tuple, list)):
            comps = [np.asarray(c) for c in val]
            for c in comps:
                if c.shape != (nx, ny, nz):
                    raise ValueError("%s: shape %s != %s" % (name, c.shape, (nx, ny, nz)))
            dt = comps[0].dtype
            stacked = np.stack([c.ravel(order="F") for c in comps], axis=1).astype(dt)
            off = add_block(np.ascontiguousarray(stacked).tobytes())
            arrays_xml.append('<DataArray type="%s" Name="%s" NumberOfComponents="3" format="appended" offset="%d"/>'
                              % (_VTK_TYPES[dt], name, off))
        else:
            a = np.asarray(val)
            if a.shape != (nx, ny, nz):
                raise ValueError("%s: shape %s != %s" % (name, a.shape, (nx, ny, nz)))
            off = add_block(np.ascontiguousarray(a.ravel(order="F")).tobytes())
            arrays_xml.append('<DataArray type="%s" Name="%s" NumberOfComponents="1" format="appended" offset="%d"/>'
                              % (_VTK_TYPES[a.dtype], name, off))
    coord_xml = []
    for name, a in (("x_coordinates", x), ("y_coordinates", y), ("z_coordinates", z)):
        off = add_block(a.tobytes())
        coord_xml.append('<DataArray type="Float64" Name="%s" NumberOfComponents="1" format="appended" offset="%d"/>'
                         % (name, off))
    extent = "0 %d 0 %d 0 %d" % (nx - 1, ny - 1, nz - 1)
    head = ('<?xml version="1.0"?>\n'
            '<VTKFile type="RectilinearGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">\n'
            '<RectilinearGrid WholeExtent="%s">\n<Piece Extent="%s">\n<PointData>\n%s\n</PointData>\n'
            '<Coordinates>\n%s\n</Coordinates>\n</Piece>\n</RectilinearGrid>\n'
            '<AppendedData encoding="raw">\n_' % (extent, extent, "\n".join(arrays_xml), "\n".join(coord_xml)))
    fname = path + ".vtr"
    with open(fname, "wb") as fh:
        fh.write(head.encode())
        for b in blocks:
            fh.write(b)
        fh.write(b"\n</AppendedData>\n</VTKFile>\n")
    return fname


def read_vtr(fname):
    """Read back a file written by grid_to_vtk (for tests): name -> array."""
    import re
    data = open(fname, "rb").read()
    head, _, tail = data.partition(b'<AppendedData encoding="raw">\n_')
    text = head.decode()
    ext = [int(t) for t in re.search(r'WholeExtent="([^"]+)"', text).group(1).split()]
    shape = (ext[1] + 1, ext[3] + 1, ext[5] + 1)
    inv = {v: k for k, v in _VTK_TYPES.items()}
    out = {}
    for m in re.finditer(r'<DataArray type="(\w+)" Name="(\w+)" NumberOfComponents="(\d)" format="appended" '
                         r'offset="(\d+)"/>', text):
        typ, name, nc, off = m.group(1), m.group(2), int(m.group(3)), int(m.group(4))
        n = int(np.frombuffer(tail[off:off + 8], np.uint64)[0])
        a = np.frombuffer(tail[off + 8:off + 8 + n], inv[typ])
        if name.endswith("_coordinates"):
            out[name] = a
        elif nc == 1:
            out[name] = a.reshape(shape, order="F")
        else:
            out[name] = a.reshape((-1, 3)).reshape(shape + (3,), order="F")
    return out
