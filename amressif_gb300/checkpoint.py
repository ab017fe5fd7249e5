"""Checkpoint files in the directory layout of the reference's SaveCheckpoint /
LoadCheckpoint (utilities.cpp:792-1023), and plotfiles in the layout of its
Export_Flow_Field (utilities.cpp:534-570, AMReX WriteSingleLevelPlotfile), host
side, for 2D and 3D states.

Layout written:

    checkpointNNNNN/Header             title line, time, cell BoxArray
    checkpointNNNNN/Level_0/<f>_H      multifab header
    checkpointNNNNN/Level_0/<f>_D_00000  one binary FAB per box
    f in pressure, vel_xCont, vel_yCont, vel_xContPrev, vel_yContPrev and,
    in 3D, vel_zCont, vel_zContPrev (utilities.cpp:821-822, 832-833, 888-889)

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

Arrays are dense numpy arrays indexed [k, j, i] (3D) or [j, i] (2D), x
fastest: the face array of direction d has n + 1 entries along d.
"""
import itertools
import os
import re

import numpy as np

TITLE = "Checkpoint file for AMRESSIF"
AXES = "xyz"
# IEEE double, little-endian byte order
REAL_DESCRIPTOR = "((8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1)))"


def fields(dim):
    """the checkpoint's multifab names, in the order SaveCheckpoint writes them"""
    return ("pressure",) + tuple("vel_%sCont" % a for a in AXES[:dim]) + tuple("vel_%sContPrev" % a for a in AXES[:dim])


def chop(n_cell, max_grid_size, dim=2):
    """Cell boxes (lo, hi) of the n^dim domain, at most max_grid_size cells per
    direction, x varying fastest."""
    per_dir = [[(a, min(a + max_grid_size[d], n_cell) - 1) for a in range(0, n_cell, max_grid_size[d])]
               for d in range(dim)]
    out = []
    for combo in itertools.product(*reversed(per_dir)):  # slowest direction outermost
        seg = list(reversed(combo))
        out.append((tuple(s[0] for s in seg), tuple(s[1] for s in seg)))
    return out


def _tup(v):
    return "(" + ",".join("%d" % x for x in v) + ")"


def _box_str(lo, hi, typ):
    return "(%s %s %s)" % (_tup(lo), _tup(hi), _tup(typ))


def _boxarray_str(boxes, typ):
    lines = ["(%d 0" % len(boxes)] + [_box_str(lo, hi, typ) for lo, hi in boxes] + [")"]
    return "\n".join(lines)


def _face_type(dim, d):
    return tuple(1 if e == d else 0 for e in range(dim))


def _field_boxes(cell_boxes, typ):
    """surroundingNodes along the nodal direction"""
    return [(lo, tuple(h + t for h, t in zip(hi, typ))) for lo, hi in cell_boxes]


def _sl(lo, hi):
    """numpy slice of the box [lo, hi] in an array indexed slowest first"""
    return tuple(slice(lo[d], hi[d] + 1) for d in reversed(range(len(lo))))


def _write_multifab(prefix, arr, boxes, typ):
    """arr: the whole field, indexed slowest direction first"""
    name = os.path.basename(prefix)
    data_name = name + "_D_00000"
    offsets, mins, maxs = [], [], []
    with open(prefix + "_D_00000", "wb") as f:
        for lo, hi in boxes:
            offsets.append(f.tell())
            sub = np.ascontiguousarray(arr[_sl(lo, hi)], dtype="<f8")
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


_BOX_RE = re.compile(r"\(\((-?\d+(?:,-?\d+)*)\) \((-?\d+(?:,-?\d+)*)\) \((\d+(?:,\d+)*)\)\)")


def _parse_boxes(text):
    return [(tuple(int(x) for x in m[0].split(",")), tuple(int(x) for x in m[1].split(",")))
            for m in _BOX_RE.findall(text)]


def _read_fab(f, off):
    f.seek(int(off))
    line = f.readline().decode()
    if not line.startswith("FAB "):
        raise ValueError("bad FAB record")
    m = _BOX_RE.search(line)
    lo = tuple(int(x) for x in m.group(1).split(","))
    hi = tuple(int(x) for x in m.group(2).split(","))
    ncomp = int(line.rsplit(" ", 1)[1])
    shape = tuple(hi[d] - lo[d] + 1 for d in reversed(range(len(lo))))
    vals = np.frombuffer(f.read(8 * int(np.prod(shape)) * ncomp), dtype="<f8")
    return lo, hi, ncomp, vals.reshape((ncomp,) + shape)


def _read_multifab(prefix, shape):
    with open(prefix + "_H") as h:
        text = h.read()
    boxes = _parse_boxes(text)
    fods = re.findall(r"FabOnDisk: (\S+) (\d+)", text)
    if len(fods) != len(boxes):
        raise ValueError("%s_H: %d boxes but %d FabOnDisk entries" % (prefix, len(boxes), len(fods)))
    out = np.full(shape, np.nan)
    d = os.path.dirname(prefix)
    for (fname, off) in fods:
        with open(os.path.join(d, fname), "rb") as f:
            lo, hi, _, vals = _read_fab(f, off)
        out[_sl(lo, hi)] = vals[0]
    if np.isnan(out).any():
        raise ValueError("%s: the boxes do not cover the field" % prefix)
    return out


def checkpoint_name(step):
    return "checkpoint%05d" % step


def write_checkpoint(root, step, u, u_prev, p, time, max_grid_size):
    """Write the state in the reference's layout under root; returns the path.
    u, u_prev: the face arrays of the dim directions; p: the cell array."""
    dim = p.ndim
    n = p.shape[0]
    path = os.path.join(root, checkpoint_name(step))
    os.makedirs(os.path.join(path, "Level_0"), exist_ok=True)
    cells = chop(n, max_grid_size, dim)
    with open(os.path.join(path, "Header"), "w") as h:
        h.write(TITLE + "\n")
        h.write("%.15g\n" % time)  # HeaderFile.precision(15), utilities.cpp:869
        h.write(_boxarray_str(cells, (0,) * dim) + "\n")
    lv = os.path.join(path, "Level_0")
    _write_multifab(os.path.join(lv, "pressure"), p, cells, (0,) * dim)
    for prev, arrs in ((False, u), (True, u_prev)):
        for d in range(dim):
            typ = _face_type(dim, d)
            name = "vel_%sCont%s" % (AXES[d], "Prev" if prev else "")
            _write_multifab(os.path.join(lv, name), arrs[d], _field_boxes(cells, typ), typ)
    return path


def read_checkpoint(path):
    """(u, u_prev, p, time) of a checkpoint directory (2D or 3D)."""
    with open(os.path.join(path, "Header")) as h:
        title = h.readline().rstrip("\n")
        if title != TITLE:
            raise ValueError("not an AMRESSIF checkpoint: %r" % title)
        time = float(h.readline())
        rest = h.read()
    cells = _parse_boxes(rest)
    dim = len(cells[0][0])
    n = max(hi[0] for _, hi in cells) + 1
    lv = os.path.join(path, "Level_0")
    p = _read_multifab(os.path.join(lv, "pressure"), (n,) * dim)

    def face(d, prev):
        shape = tuple(n + (1 if e == d else 0) for e in reversed(range(dim)))
        return _read_multifab(os.path.join(lv, "vel_%sCont%s" % (AXES[d], "Prev" if prev else "")), shape)

    u = [face(d, False) for d in range(dim)]
    up = [face(d, True) for d in range(dim)]
    return u, up, p, time


# ---- plotfiles (Export_Flow_Field) ----------------------------------------------------

def plot_vars(dim):
    return ("pressure", "U", "V", "W")[: dim + 1]


def cell_velocity(u):
    """velCart of cont2cart (utilities.cpp:49-53): face averages at the cells
    (host restatement; Solver.cell_velocity computes it on the device)"""
    dim = len(u)
    out = []
    for d in range(dim):
        ax = dim - 1 - d  # numpy axis of direction d
        a = np.moveaxis(u[d], ax, 0)
        out.append(np.moveaxis(0.5 * (a[:-1] + a[1:]), 0, ax))
    return out


def write_plotfile(root, name, step, u, p, time, max_grid_size, prob_lo=None, prob_hi=None, cart=None):
    """pltfile <name>NNNNN with the components pressure, U, V (and W in 3D),
    as Export_Flow_Field writes them; cart: the cell velocity (default: the
    face averages of u); returns the path."""
    dim = p.ndim
    n = p.shape[0]
    prob_lo = tuple(prob_lo) if prob_lo is not None else (0.0,) * dim
    prob_hi = tuple(prob_hi) if prob_hi is not None else (1.0,) * dim
    path = os.path.join(root, "%s%05d" % (name, step))
    os.makedirs(os.path.join(path, "Level_0"), exist_ok=True)
    cells = chop(n, max_grid_size, dim)
    dx = [(prob_hi[d] - prob_lo[d]) / n for d in range(dim)]
    comps = [p] + list(cart if cart is not None else cell_velocity(u))
    names = plot_vars(dim)
    z = (0,) * dim
    with open(os.path.join(path, "Header"), "w") as h:
        h.write("HyperCLaw-V1.1\n%d\n" % len(names))
        h.write("".join(v + "\n" for v in names))
        h.write("%d\n%.17g\n0\n" % (dim, time))
        h.write(" ".join("%.17g" % x for x in prob_lo) + "\n")
        h.write(" ".join("%.17g" % x for x in prob_hi) + "\n\n")
        h.write(_box_str(z, (n - 1,) * dim, z) + "\n")
        h.write("%d\n%s\n0\n0\n" % (step, " ".join("%.17g" % x for x in dx)))
        h.write("0 %d %.17g\n%d\n" % (len(cells), time, step))
        for lo, hi in cells:
            for d in range(dim):
                h.write("%.17g %.17g\n" % (prob_lo[d] + lo[d] * dx[d], prob_lo[d] + (hi[d] + 1) * dx[d]))
        h.write("Level_0/Cell\n")
    prefix = os.path.join(path, "Level_0", "Cell")
    offsets, mins, maxs = [], [], []
    with open(prefix + "_D_00000", "wb") as f:
        for lo, hi in cells:
            offsets.append(f.tell())
            f.write(("FAB %s%s %d\n" % (REAL_DESCRIPTOR, _box_str(lo, hi, z), len(comps))).encode())
            for c in comps:  # component-major, Fortran order within a component
                f.write(np.ascontiguousarray(c[_sl(lo, hi)], dtype="<f8").tobytes())
            mins.append([float(c[_sl(lo, hi)].min()) for c in comps])
            maxs.append([float(c[_sl(lo, hi)].max()) for c in comps])
    with open(prefix + "_H", "w") as h:
        h.write("1\n0\n%d\n0\n" % len(comps))
        h.write(_boxarray_str(cells, z) + "\n")
        h.write("%d\n" % len(cells))
        for off in offsets:
            h.write("FabOnDisk: Cell_D_00000 %d\n" % off)
        for table in (mins, maxs):
            h.write("\n%d,%d\n" % (len(cells), len(comps)))
            h.write("".join("".join("%.17g," % v for v in row) + "\n" for row in table))
    return path


def read_plotfile(path):
    """{variable: cell array}, time and step of a plotfile written above"""
    with open(os.path.join(path, "Header")) as h:
        lines = h.read().splitlines()
    nv = int(lines[1])
    names = lines[2:2 + nv]
    dim = int(lines[2 + nv])
    time = float(lines[3 + nv])
    with open(os.path.join(path, "Level_0", "Cell_H")) as h:
        text = h.read()
    boxes = _parse_boxes(text)
    fods = re.findall(r"FabOnDisk: (\S+) (\d+)", text)
    n = max(hi[0] for _, hi in boxes) + 1
    out = {v: np.full((n,) * dim, np.nan) for v in names}
    for fname, off in fods:
        with open(os.path.join(path, "Level_0", fname), "rb") as f:
            lo, hi, _, vals = _read_fab(f, off)
        for k, v in enumerate(names):
            out[v][_sl(lo, hi)] = vals[k]
    step = int(lines[nv + 9])  # after the domain box of level 0
    return out, time, step
