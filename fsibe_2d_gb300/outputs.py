"""The reference's per-step text files, written from the records of fsibe_run_records.

Per time step the reference appends one line to each of these files in dir_name (with the
simulation name as a prefix), each with its own Fortran format:

    beam_data<i>  '(21(es15.8,1x))'    BeamIO.f90:193-216 (SaveBeamData, iSaveBeam = 3)
    u_max         '(1x,5(es12.4,1x))'  NavierStokes.f90:80-82 (cal_nlk)
    energies      '(8(es15.8,1x))'     NavierStokes.f90:259-261 (cal_energy)
    IBES_iter     '(es11.4,1x,i3)'     SolidSolver.f90:392-394 (IBES_solver, iFLUSI = 1)
    mouvement<i>  '(10(es15.8,1x))'    BeamIO.f90:229-238 (SaveBeamData, every step)

A record (FSIBE_RECORD_COLS values) holds the five rows of one step in that order; the
column layout is documented at fsibe_run_records in include/fsibe.h.  The files are opened
in append mode, as the reference opens them (status='unknown', access='append')."""
import math
import os

import numpy as np

from ._abi import FSIBE_RECORD_COLS

BEAM = slice(0, 21)
UMAX = slice(21, 26)
ENERGIES = slice(26, 34)
IBES = slice(34, 36)
MOUVEMENT = slice(36, 46)


def es(v, w, d):
    """Fortran ESw.d edit of a real: one non-zero digit before the point, d after it, a signed
    two-digit exponent after 'E' (three digits, without the 'E', beyond 99), right-justified
    in w characters; asterisks when it does not fit."""
    v = float(v)
    if math.isnan(v):
        s = "NaN"
    elif math.isinf(v):
        s = "Infinity" if v > 0 else "-Infinity"
        if len(s) > w:
            s = "Inf" if v > 0 else "-Inf"
    else:
        mant, exp = f"{v:.{d}E}".split("E")
        e = int(exp)
        s = mant + ("E%+03d" % e if abs(e) <= 99 else "%+04d" % e)
    return s.rjust(w) if len(s) <= w else "*" * w


def beam_data_line(row):
    return "".join(es(v, 15, 8) + " " for v in row)


def u_max_line(row):
    return " " + "".join(es(v, 12, 4) + " " for v in row)


def energies_line(row):
    return "".join(es(v, 15, 8) + " " for v in row)


def mouvement_line(row):
    return "".join(es(v, 15, 8) + " " for v in row)


def ibes_iter_line(row):
    it = int(round(row[1]))
    return es(row[0], 11, 4) + " " + ("%3d" % it if -99 <= it <= 999 else "***")


def write_step_files(directory, records, simulation_name="", beam=1, iFLUSI=1, iSaveBeam=3, t_release=0.0):
    """Append the lines of every record to the reference's per-step files in directory.
    beam_data<beam> is written when iSaveBeam = 3 and IBES_iter when iFLUSI = 1, for the steps
    that start after t_release (SolidSolverWrapper calls IBES_solver only then,
    SolidSolver.f90:20-27); u_max, energies and mouvement<beam> every step.  Returns the paths written."""
    rec = np.asarray(records, dtype=np.float64).reshape(-1, FSIBE_RECORD_COLS)
    os.makedirs(directory, exist_ok=True)
    base = os.path.join(directory, simulation_name)
    every = np.ones(len(rec), dtype=bool)
    files = [("u_max", UMAX, u_max_line, every), ("energies", ENERGIES, energies_line, every)]
    if iSaveBeam == 3:
        files.insert(0, (f"beam_data{beam}", BEAM, beam_data_line, every))
    if iFLUSI == 1:
        files.append(("IBES_iter", IBES, ibes_iter_line, rec[:, IBES.start] > t_release))
    files.append((f"mouvement{beam}", MOUVEMENT, mouvement_line, every))
    paths = []
    for name, cols, fmt, which in files:
        path = base + name
        with open(path, "a") as f:
            for r in rec[which]:
                f.write(fmt(r[cols]) + "\n")
        paths.append(path)
    return paths


def write_field(filename, field, nsave=1, lx=None, ly=None, fieldtype="pressure", header=()):
    """SaveField (FieldExport.f90:612-648), '%format1': the header lines (the reference writes its
    PARAMS file there; pass them as `header`), '%format1', nx and ny of the field as i5.5, the
    domain sizes as es11.4, the type line, then one value a line, es11.4 (es16.9 for the type
    "precision"): rows from the top (y index ny - 1) down in steps of nsave, each row from
    x index 0 in steps of nsave.  field: (ny, nx), the layout of the library's fields."""
    f = np.asarray(field, dtype=np.float64)
    ny1, nx1 = f.shape
    fmt = (lambda v: es(v, 16, 9)) if fieldtype == "precision" else (lambda v: es(v, 11, 4))
    lines = list(header)
    lines += ["%format1", "%05d   %% nx" % nx1, "%05d   %% ny" % ny1,
              es(lx, 11, 4) + "   % xl, domain size in x-direction",
              es(ly, 11, 4) + "   % yl, domain size in y-direction",
              "% The next entry can be used to identify the type of the field: ",
              "% " + fieldtype]
    for iy in range(0, ny1, nsave):
        row = f[ny1 - 1 - iy]
        lines += [fmt(v) for v in row[0:nx1:nsave]]
    with open(filename, "w") as out:
        out.write("\n".join(lines) + "\n")
    return filename
