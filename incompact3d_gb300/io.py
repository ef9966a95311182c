"""File formats of the reference around the time step.

* ``time_evol.dat`` of the TGV case (src/Case-TGV.f90:375-377): one row per
  statistics step, ``(20e20.12)`` in double precision and ``(14e14.6)`` in
  single precision; ``fortran_e`` reproduces the Fortran ``Ew.d`` edit
  descriptor so rows diff against the reference's own files.
* The ``.i3d`` input namelists (src/parameters.f90:40-340): ``read_namelist``
  parses ``&Group ... /End`` blocks; ``case_from_i3d`` maps the subset this
  package implements to Context / Solver arguments.
* Restart files (restart, src/tools.f90:205-514): the variables are written
  one after the other as whole global arrays in Fortran order (x fastest,
  binary64, native byte order) into one file -- ux, uy, uz, the AB history
  (dux-2..duz-2 for AB2/AB3, dux-3..duz-3 for AB3) and pp on the pressure
  mesh -- plus the ``restart.info`` namelist (&Time, &NumParam).
"""
import ctypes
import math
import os
import re

import numpy as np

from ._lib import check


# --------------------------------------------------------------------------
# Fortran Ew.d
# --------------------------------------------------------------------------
def fortran_e(v, w=20, d=12):
    """``Ew.d`` output of one real, right-justified in w characters:
    0.ddd...dE+xx (three-digit exponents drop the E, as Fortran does)."""
    v = float(v)
    if math.isnan(v):
        s = "NaN"
    elif math.isinf(v):
        s = "Infinity" if v > 0 else "-Infinity"
    elif v == 0.0:
        s = ("-" if math.copysign(1.0, v) < 0 else "") + "0." + "0" * d + "E+00"
    else:
        # d significant digits: mantissa in [0.1, 1) after rounding
        m = "{:.{p}E}".format(abs(v), p=d - 1)   # D.DDDDE+xx
        digits, ex = m.split("E")
        digits = digits.replace(".", "")
        e = int(ex) + 1
        sign = "-" if v < 0 else ""
        if abs(e) <= 99:
            es = "E{}{:02d}".format("+" if e >= 0 else "-", abs(e))
        else:
            es = "{}{:03d}".format("+" if e >= 0 else "-", abs(e))
        s = sign + "0." + digits + es
    return s.rjust(w)


def format_time_evol_row(row, double=True):
    """One row (t, E_k, eps, eps2, enstrophy) as the reference writes it."""
    w, d = (20, 12) if double else (14, 6)
    return "".join(fortran_e(x, w, d) for x in row)


def write_time_evol(path, rows, double=True):
    with open(path, "w") as f:
        for r in rows:
            f.write(format_time_evol_row(r, double) + "\n")


# --------------------------------------------------------------------------
# .i3d namelists
# --------------------------------------------------------------------------
def _value(tok):
    t = tok.strip()
    low = t.lower()
    if low in (".true.", "t", "true", ".t."):
        return True
    if low in (".false.", "f", "false", ".f."):
        return False
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "'\"":
        return t[1:-1]
    num = low.replace("d", "e") if re.fullmatch(r"[+-]?[0-9.]+[de][+-]?[0-9]+", low) else low
    try:
        if re.fullmatch(r"[+-]?[0-9]+", num):
            return int(num)
        return float(num)
    except ValueError:
        return t


def read_namelist(text):
    """Parse Fortran namelist groups: {group_lower: {key_lower: value}}.
    Comments start with '!'; values are int, float, logical or string; array
    entries (key(i) = v) are kept under 'key(i)'."""
    groups = {}
    cur = None
    for raw in text.splitlines():
        line = raw.split("!", 1)[0].strip()
        if not line:
            continue
        if line.startswith("&"):
            name = line[1:].strip().lower()
            if name in ("end", ""):
                cur = None
                continue
            cur = groups.setdefault(name, {})
            continue
        if line.startswith("/"):
            cur = None
            continue
        if cur is None:
            continue
        for part in re.split(r",(?=\s*[A-Za-z_][A-Za-z0-9_()]*\s*=)", line):
            if "=" not in part:
                continue
            k, v = part.split("=", 1)
            v = v.strip().rstrip(",")
            vals = [x for x in re.split(r"[,\s]+", v) if x] if not v.startswith(("'", '"')) else [v]
            cur[k.strip().lower()] = _value(vals[0]) if len(vals) == 1 else [_value(x) for x in vals]
    return groups


# itype values of src/module_param.f90 used here
ITYPE_TGV, ITYPE_CHANNEL = 2, 3


def case_from_i3d(path_or_text):
    """Context, Solver and case settings from an input namelist, for the subset
    implemented here (grid, BCs, stretching, schemes, time scheme, LES model,
    channel forcing).  Returns a dict with keys 'context' (Context kwargs),
    'solver' (Solver kwargs), 'itype', 'les' (jles, smagcst, maxdsmagcst) and
    'channel' (wrotation, spinup_time)."""
    text = open(path_or_text).read() if os.path.exists(str(path_or_text)) else str(path_or_text)
    g = read_namelist(text)
    b = g.get("basicparam", {})
    n = g.get("numoptions", {})
    les = g.get("lesmodel", {})
    st = g.get("statistics", {})
    get = lambda d, k, dv: d.get(k, dv)  # noqa: E731
    ctx = dict(nx=int(b["nx"]), ny=int(b["ny"]), nz=int(b["nz"]),
               xlx=float(b["xlx"]), yly=float(b["yly"]), zlz=float(b["zlz"]),
               bc=((int(get(b, "nclx1", 0)), int(get(b, "nclxn", 0))),
                   (int(get(b, "ncly1", 0)), int(get(b, "nclyn", 0))),
                   (int(get(b, "nclz1", 0)), int(get(b, "nclzn", 0)))),
               ifirstder=int(get(n, "ifirstder", 4)), isecondder=int(get(n, "isecondder", 4)),
               ipinter=int(get(n, "ipinter", 3)), nu0nu=float(get(n, "nu0nu", 4.0)),
               cnu=float(get(n, "cnu", 0.44)), istret=int(get(b, "istret", 0)),
               beta=float(get(b, "beta", 0.0)))
    if "c_filter" in b:
        ctx["filter_alpha"] = float(b["c_filter"])  # filter(C_filter), src/parameters.f90:788
    solver = dict(dt=float(b["dt"]), xnu=1.0 / float(b["re"]), itimescheme=int(get(n, "itimescheme", 3)))
    jles = int(get(les, "jles", 0)) if int(get(b, "ilesmod", 0)) != 0 else 0
    return {"context": ctx, "solver": solver, "itype": int(get(b, "itype", ITYPE_TGV)),
            "les": (jles, float(get(les, "smagcst", 0.15)), float(get(les, "maxdsmagcst", 0.3))),
            "channel": (float(get(st, "wrotation", 0.0)), int(get(st, "spinup_time", 0))),
            "steps": (int(get(b, "ifirst", 1)), int(get(b, "ilast", 1)))}


# --------------------------------------------------------------------------
# restart files
# --------------------------------------------------------------------------
_AB_SLOTS = {2: (3, 4, 5), 3: (3, 4, 5, 6, 7, 8)}


def _fortran_f(v, w, d):
    return ("{:.%df}" % d).format(v).rjust(w)


def write_restart(directory, solver, t, itime):
    """Write ``restart`` (the fields, one global array after the other in the
    reference's order) and ``restart.info`` for the solver's state."""
    os.makedirs(directory, exist_ok=True)
    ctx = solver.ctx
    nx, ny, nz = ctx.n
    ts = solver.itimescheme
    slots = [0, 1, 2] + list(_AB_SLOTS.get(ts, ())) + [9]
    with open(os.path.join(directory, "restart"), "wb") as f:
        for w in slots:
            a = solver.get_field(w)
            f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
    lines = ["!=========================", "&Time", "!=========================",
             "tfield=   " + _fortran_f(t, 16, 4), "itime=    " + str(itime).rjust(16), "/End",
             "!=========================", "&NumParam", "!=========================",
             "nx=       " + str(nx).rjust(16), "ny=       " + str(ny).rjust(16), "nz=       " + str(nz).rjust(16),
             "Lx=       " + _fortran_f(ctx.L[0], 16, 4), "Ly=       " + _fortran_f(ctx.L[1], 16, 4),
             "Lz=       " + _fortran_f(ctx.L[2], 16, 4), "istret=   " + str(ctx.istret).rjust(16),
             "beta=     " + _fortran_f(ctx.beta, 16, 12), "iscalar=  " + "0".rjust(16),
             "numscalar=" + "0".rjust(16), "itimescheme=" + str(ts).rjust(14), "iimplicit=" + "0".rjust(16),
             "/End", "!========================="]
    with open(os.path.join(directory, "restart.info"), "w") as f:
        f.write("\n".join(lines) + "\n")


def read_restart(directory, solver):
    """Load a restart written by ``write_restart`` (or by the reference's
    MPI-IO writer for the same variables) into the solver; returns
    (t, itime) from ``restart.info``."""
    info = read_namelist(open(os.path.join(directory, "restart.info")).read())
    t = float(info["time"]["tfield"])
    itime = int(info["time"]["itime"])
    ctx = solver.ctx
    nx, ny, nz = ctx.n
    N = nx * ny * nz
    nxm, nym, nzm = ctx.nm
    ts = int(info["numparam"].get("itimescheme", solver.itimescheme))
    if ts != solver.itimescheme:
        raise ValueError("restart written with itimescheme=%d, solver uses %d" % (ts, solver.itimescheme))
    raw = np.fromfile(os.path.join(directory, "restart"), dtype=np.float64)
    slots = [0, 1, 2] + list(_AB_SLOTS.get(ts, ()))
    need = len(slots) * N + nxm * nym * nzm
    if raw.size != need:
        raise ValueError("restart holds %d values, expected %d" % (raw.size, need))
    off = 0
    for w in slots:
        solver.set_field(w, raw[off:off + N].reshape(nz, ny, nx))
        off += N
    solver.set_field(9, raw[off:].reshape(nzm, nym, nxm))
    solver.set_itime(itime)
    return t, itime
