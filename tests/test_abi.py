"""The C-ABI library loads here (no GPU needed) and exports every entry point include/fsibe.h
declares; the ctypes structs match the C layout compiled from the header."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "fsibe.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(fsibe_\w+)\s*\(", text, re.M)))


def test_library_loads_and_exports_every_declared_symbol():
    import fsibe_2d_gb300 as F
    from fsibe_2d_gb300 import build as b
    b.build()
    lib = F.library()
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.fsibe_strerror(0) == b"ok"


def test_oracle_exports_the_same_entry_points(oracle):
    lib = oracle.lib()
    skip = {"fsibe_set_stream", "fsibe_strerror", "fsibe_time_steps", "fsibe_launches_per_step", "fsibe_use_graph",
            "fsibe_kernel_times", "fsibe_coftxy_static", "fsibe_beam_phase_cycles",
            "fsibe_ensemble_create", "fsibe_ensemble_destroy", "fsibe_ensemble_size", "fsibe_ensemble_get",
            "fsibe_ensemble_step", "fsibe_ensemble_time_steps", "fsibe_ensemble_last_error",
            "fsibe_drag_objective", "fsibe_drag_gradient", "fsibe_force_objective", "fsibe_force_gradient",
            "fsibe_tiles", "fsibe_tile_config", "fsibe_beam_cluster", "fsibe_press_y_engine", "fsibe_running_sums",
            "fsibe_last_error"}
    missing = [n for n in declared_functions() if n not in skip and not hasattr(lib, "orc_" + n[len("fsibe_"):])]
    assert not missing, missing


def test_ctypes_structs_match_the_c_layout():
    from fsibe_2d_gb300._abi import FsibeParams, FsibeScalars
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "fsibe.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(fsibe_params), sizeof(fsibe_scalars),
         offsetof(fsibe_params, newton_tol), offsetof(fsibe_scalars, beam_data),
         offsetof(fsibe_params, N_smooth), offsetof(fsibe_scalars, newton_iters));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe])
        vals = [int(v) for v in subprocess.check_output([exe]).split()]
    assert vals == [C.sizeof(FsibeParams), C.sizeof(FsibeScalars), FsibeParams.newton_tol.offset,
                    FsibeScalars.beam_data.offset, FsibeParams.N_smooth.offset, FsibeScalars.newton_iters.offset]


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    import fsibe_2d_gb300 as F
    monkeypatch.setattr(F, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(F, "_lib", None)
    with pytest.raises(RuntimeError):
        F.library()
