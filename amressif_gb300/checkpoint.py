"""Checkpoint files in the directory layout of the reference's SaveCheckpoint /
LoadCheckpoint (utilities.cpp:792-1023), and plotfiles in the layout of its
Export_Flow_Field (utilities.cpp:534-570, AMReX WriteSingleLevelPlotfile), host
side.

Layout written (2D):

    checkpointNNNNN/Header             title line, time, cell BoxArray
    checkpointNNNNN/Level_0/<f>_H      multifab header
    checkpointNNNNN/Level_0/<f>_D_00000  one binary FAB per box
    f in pressure, vel_xCont, vel_yCont, vel_xContPrev, vel_yContPrev

The BoxArray is the domain chopped into boxes of at most max_grid_size cells
per direction (the reference's ba.maxSize). Face MultiFabs use the
surrounding-nodes boxes (type 1 along the face direction). The multifab
header and FAB records follow AMReX's documented VisMF text/binary layout
(header version 1, one data file, FAB records "FAB <real descriptor><box>
<ncomp>" followed by the values in Fortran order as IEEE doubles); the format
is restated from that documentation and has not been checked against an
AMReX build, which is not available here. phi is not saved, as in the
reference; the state (u^n, u^{n-1}, p, time) is what ns_checkpoint_put needs
for a bit-exact restart.
"""
import os
import re

import numpy as np

TITLE = "Checkpoint file for AMRESSIF"
FIELDS = ("pressure", "vel_xCont", "vel_yCont", "vel_xContPrev", "vel_yContPrev")
# IEEE double, little-endian byte order
REAL_DESCRIPTOR = "((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))"


def chop(n_cell, max_grid_size):
    """Cell boxes (lo, hi) of the n x n domain, at most max_grid_size per
    direction, x varying fastest."""
    mx, my = max_grid_size[0], max_grid_size[1]
    xs = [(a, min(a + mx, n_cell) - 1) for a in range(0, n_cell, mx)]
    ys = [(b, min(b + my, n_cell) - 1) for b in range(0, n_cell, my)]
    return [((x0, y0), (x1, y1)) for (y0, y1) in ys for (x0, x1) in xs]


def _box_str(lo, hi, typ):
    return "((%d,%d) (%d,%d) (%d,%d))" % (lo[0], lo[1], hi[0], hi[1], typ[0], typ[1])


def _boxarray_str(boxes, typ):
    lines = ["(%d 0" % len(boxes)] + [_box_str(lo, hi, typ) for lo, hi in boxes] + [")"]
    return "\n".join(lines)


def _field_boxes(cell_boxes, typ):
    """surroundingNodes along the nodal direction"""
    out = []
    for lo, hi in cell_boxes:
        hi2 = (hi[0] + typ[0], hi[1] + typ[1])
        out.append((lo, hi2))
    return out


def _write_multifab(prefix, arr, boxes, typ):
    """arr: dense (rows = y, cols = x) array of the whole field"""
    name = os.path.basename(prefix)
    data_name = name + "_D_00000"
    offsets, mins, maxs = [], [], []
    with open(prefix + "_D_00000", "wb") as f:
        for lo, hi in boxes:
            offsets.append(f.tell())
            sub = np.ascontiguousarray(arr[lo[1]:hi[1] + 1, lo[0]:hi[0] + 1], dtype="<f8")
            f.write(("FAB %s%s 1\n" % (REAL_DESCRIPTOR, _box_str(lo, hi, typ))).encode())
            f.write(sub.tobytes())
            mins.append(float(sub.min()))
            maxs.append(float(sub.max()))
    with open(prefix + "_H", "w") as h:
        h.write("1\n0\n1\n0\n")
        h.write(_boxarray_str(boxes, typ) + "\n")
        h.write("%d\n" % len(boxes))
        for off in offsets:
            h.write("FabOnDisk: %s %d\n" % (data_name, off))
        h.write("\n%d,1\n" % len(boxes))
        h.write("".join("%.17g,\n" % v for v in mins))
        h.write("\n%d,1\n" % len(boxes))
        h.write("".join("%.17g,\n" % v for v in maxs))


_BOX_RE = re.compile(r"\(\((-?\d+),(-?\d+)\) \((-?\d+),(-?\d+)\) \((\d+),(\d+)\)\)")


def _read_multifab(prefix, shape):
    with open(prefix + "_H") as h:
        text = h.read()
    boxes = [((int(m[0]), int(m[1])), (int(m[2]), int(m[3]))) for m in _BOX_RE.findall(text)]
    fods = re.findall(r"FabOnDisk: (\S+) (\d+)", text)
    if len(fods) != len(boxes):
        raise ValueError("%s_H: %d boxes but %d FabOnDisk entries" % (prefix, len(boxes), len(fods)))
    out = np.full(shape, np.nan)
    d = os.path.dirname(prefix)
    for (lo, hi), (fname, off) in zip(boxes, fods):
        with open(os.path.join(d, fname), "rb") as f:
            f.seek(int(off))
            line = f.readline().decode()
            if not line.startswith("FAB "):
                raise ValueError("bad FAB record in %s" % fname)
            m = _BOX_RE.search(line)
            blo, bhi = (int(m[1]), int(m[2])), (int(m[3]), int(m[4]))
            ncomp = int(line.rsplit(" ", 1)[1])
            nx, ny = bhi[0] - blo[0] + 1, bhi[1] - blo[1] + 1
            vals = np.frombuffer(f.read(8 * nx * ny * ncomp), dtype="<f8")
            out[blo[1]:bhi[1] + 1, blo[0]:bhi[0] + 1] = vals[: nx * ny].reshape(ny, nx)
    if np.isnan(out).any():
        raise ValueError("%s: the boxes do not cover the field" % prefix)
    return out


def checkpoint_name(step):
    return "checkpoint%05d" % step


def write_checkpoint(root, step, u, u_prev, p, time, max_grid_size):
    """Write the state in the reference's layout under root; returns the path.
    u, u_prev: [u (n, n+1), v (n+1, n)]; p: (n, n)."""
    n = p.shape[0]
    path = os.path.join(root, checkpoint_name(step))
    os.makedirs(os.path.join(path, "Level_0"), exist_ok=True)
    cells = chop(n, max_grid_size)
    with open(os.path.join(path, "Header"), "w") as h:
        h.write(TITLE + "\n")
        h.write("%.15g\n" % time)
        h.write(_boxarray_str(cells, (0, 0)) + "\n")
    lv = os.path.join(path, "Level_0")
    _write_multifab(os.path.join(lv, "pressure"), p, cells, (0, 0))
    for name, arr, typ in (("vel_xCont", u[0], (1, 0)), ("vel_yCont", u[1], (0, 1)),
                           ("vel_xContPrev", u_prev[0], (1, 0)), ("vel_yContPrev", u_prev[1], (0, 1))):
        _write_multifab(os.path.join(lv, name), arr, _field_boxes(cells, typ), typ)
    return path


def read_checkpoint(path):
    """(u, u_prev, p, time) of a checkpoint directory."""
    with open(os.path.join(path, "Header")) as h:
        title = h.readline().rstrip("\n")
        if title != TITLE:
            raise ValueError("not an AMRESSIF checkpoint: %r" % title)
        time = float(h.readline())
        rest = h.read()
    cells = [((int(m[0]), int(m[1])), (int(m[2]), int(m[3]))) for m in _BOX_RE.findall(rest)]
    n = max(hi[0] for _, hi in cells) + 1
    lv = os.path.join(path, "Level_0")
    p = _read_multifab(os.path.join(lv, "pressure"), (n, n))
    u = [_read_multifab(os.path.join(lv, "vel_xCont"), (n, n + 1)), _read_multifab(os.path.join(lv, "vel_yCont"), (n + 1, n))]
    up = [_read_multifab(os.path.join(lv, "vel_xContPrev"), (n, n + 1)),
          _read_multifab(os.path.join(lv, "vel_yContPrev"), (n + 1, n))]
    return u, up, p, time


# ---- plotfiles (Export_Flow_Field) ----------------------------------------------------

PLOT_VARS = ("pressure", "U", "V")


def cell_velocity(u):
    """velCart of cont2cart (utilities.cpp:49-53): face averages at the cells"""
    return 0.5 * (u[0][:, :-1] + u[0][:, 1:]), 0.5 * (u[1][:-1, :] + u[1][1:, :])


def write_plotfile(root, name, step, u, p, time, max_grid_size, prob_lo=(0.0, 0.0), prob_hi=(1.0, 1.0)):
    """pltfile <name>NNNNN with the components pressure, U, V (cell-centred
    velocity from the faces), as Export_Flow_Field writes them; returns the path."""
    n = p.shape[0]
    path = os.path.join(root, "%s%05d" % (name, step))
    os.makedirs(os.path.join(path, "Level_0"), exist_ok=True)
    cells = chop(n, max_grid_size)
    dx = [(prob_hi[d] - prob_lo[d]) / n for d in range(2)]
    cu, cv = cell_velocity(u)
    comps = [p, cu, cv]
    with open(os.path.join(path, "Header"), "w") as h:
        h.write("HyperCLaw-V1.1\n%d\n" % len(PLOT_VARS))
        h.write("".join(v + "\n" for v in PLOT_VARS))
        h.write("2\n%.17g\n0\n" % time)
        h.write("%.17g %.17g\n%.17g %.17g\n\n" % (prob_lo[0], prob_lo[1], prob_hi[0], prob_hi[1]))
        h.write(_box_str((0, 0), (n - 1, n - 1), (0, 0)) + "\n")
        h.write("%d\n%.17g %.17g\n0\n0\n" % (step, dx[0], dx[1]))
        h.write("0 %d %.17g\n%d\n" % (len(cells), time, step))
        for lo, hi in cells:
            for d in range(2):
                h.write("%.17g %.17g\n" % (prob_lo[d] + lo[d] * dx[d], prob_lo[d] + (hi[d] + 1) * dx[d]))
        h.write("Level_0/Cell\n")
    prefix = os.path.join(path, "Level_0", "Cell")
    offsets, mins, maxs = [], [], []
    with open(prefix + "_D_00000", "wb") as f:
        for lo, hi in cells:
            offsets.append(f.tell())
            f.write(("FAB %s%s %d\n" % (REAL_DESCRIPTOR, _box_str(lo, hi, (0, 0)), len(comps))).encode())
            for c in comps:  # component-major, Fortran order within a component
                sub = np.ascontiguousarray(c[lo[1]:hi[1] + 1, lo[0]:hi[0] + 1], dtype="<f8")
                f.write(sub.tobytes())
            mins.append([float(c[lo[1]:hi[1] + 1, lo[0]:hi[0] + 1].min()) for c in comps])
            maxs.append([float(c[lo[1]:hi[1] + 1, lo[0]:hi[0] + 1].max()) for c in comps])
    with open(prefix + "_H", "w") as h:
        h.write("1\n0\n%d\n0\n" % len(comps))
        h.write(_boxarray_str(cells, (0, 0)) + "\n")
        h.write("%d\n" % len(cells))
        for off in offsets:
            h.write("FabOnDisk: Cell_D_00000 %d\n" % off)
        for table in (mins, maxs):
            h.write("\n%d,%d\n" % (len(cells), len(comps)))
            h.write("".join("".join("%.17g," % v for v in row) + "\n" for row in table))
    return path


def read_plotfile(path):
    """{variable: (n, n) array}, time and step of a plotfile written above"""
    with open(os.path.join(path, "Header")) as h:
        lines = h.read().splitlines()
    nv = int(lines[1])
    names = lines[2:2 + nv]
    time = float(lines[3 + nv])
    with open(os.path.join(path, "Level_0", "Cell_H")) as h:
        text = h.read()
    boxes = [((int(m[0]), int(m[1])), (int(m[2]), int(m[3]))) for m in _BOX_RE.findall(text)]
    fods = re.findall(r"FabOnDisk: (\S+) (\d+)", text)
    n = max(hi[0] for _, hi in boxes) + 1
    out = {v: np.full((n, n), np.nan) for v in names}
    for (lo, hi), (fname, off) in zip(boxes, fods):
        with open(os.path.join(path, "Level_0", fname), "rb") as f:
            f.seek(int(off))
            f.readline()
            nx, ny = hi[0] - lo[0] + 1, hi[1] - lo[1] + 1
            vals = np.frombuffer(f.read(8 * nx * ny * nv), dtype="<f8").reshape(nv, ny, nx)
            for k, v in enumerate(names):
                out[v][lo[1]:hi[1] + 1, lo[0]:hi[0] + 1] = vals[k]
    step = int(lines[nv + 9])  # after the domain box of level 0
    return out, time, step
