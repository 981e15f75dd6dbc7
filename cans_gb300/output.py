"""Host-side writers of the reference's text output (src/output.f90).

Every number is written with the reference's FP64 edit descriptor `es24.16e3` followed by
one blank (`fmt_dp = '(*(es24.16e3,1x))'`, src/output.f90:16-17), one record per line.
The statistics themselves come from the library's device reductions (cans_out1d,
cans_out1d_chan, cans_out2d_duct); this module only formats and writes them.
"""
import numpy as np


def es(x, w=24, d=16, e=3):
    """Fortran `ESw.dEe` of one value: one digit before the point, d after, an exponent of
    e digits with its sign, right-justified in w columns."""
    x = float(x)
    if not np.isfinite(x):
        return ("NaN" if np.isnan(x) else ("-Infinity" if x < 0 else "Infinity")).rjust(w)
    mant, ex = f"{x:.{d}E}".split("E")
    return f"{mant}E{int(ex):+0{e + 1}d}".rjust(w)


def record(values):
    return "".join(es(v) + " " for v in values)


def write_records(fname, rows, append=False):
    with open(fname, "a" if append else "w") as f:
        for r in rows:
            f.write(record(r) + "\n")


def out0d(fname, var):
    """out0d (src/output.f90:24-43): append one record."""
    write_records(fname, [var], append=True)


def write_out1d(fname, idir, ng, dl, z_g, p1d):
    """The file of out1d (src/output.f90:56-157): coordinate and average per line; the
    coordinate is z_g(k) for idir = 3 and the cell centre (i - 1/2) dl otherwise."""
    q = ng[idir - 1]
    p1d = np.asarray(p1d)
    if idir == 3:
        coord = np.asarray(z_g)[1:q + 1]
    else:
        coord = (np.arange(1, q + 1) - .5) * dl[idir - 1]
    write_records(fname, zip(coord, p1d))


def write_out1d_chan(fname, ng, z_g, stats):
    """The file of out1d_chan (src/output.f90:383-389): z, um, vm, wm, u2, v2, w2, uw."""
    st = np.asarray(stats).reshape(7, ng[2])
    z = np.asarray(z_g)[1:ng[2] + 1]
    write_records(fname, (tuple([z[k]] + list(st[:, k])) for k in range(ng[2])))


def write_out2d_duct(fname, idir, ng, dl, z_g, stats):
    """The file of out2d_duct (src/output.f90:463-472, 516-525): the cross-stream coordinate
    (cell centre), z, then the eight statistics, k slowest."""
    q = ng[1] if idir == 1 else ng[0]
    st = np.asarray(stats).reshape(8, ng[2], q)
    z = np.asarray(z_g)[1:ng[2] + 1]
    h = dl[1] if idir == 1 else dl[0]
    rows = ((tuple([(j + .5) * h, z[k]] + list(st[:, k, j]))) for k in range(ng[2]) for j in range(q))
    write_records(fname, rows)
