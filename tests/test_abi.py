"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, and its host-side logic (parameter derivation, argument checks)
behaves like the reference's setup code. No kernel runs here."""
from __future__ import annotations

import ctypes as C
import json
import re
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import fluids3_gb300 as F
from fluids3_gb300 import _lib, scenes
from oracle import oracle as O
from oracle import params_oracle as PO

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_symbols() -> set[str]:
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(fl_[a-z_0-9]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_phase_surface():
    names = declared_symbols()
    for want in ("fl_create", "fl_insert_particles", "fl_prefix_sum_cells", "fl_counting_sort_full",
                 "fl_compute_pressure", "fl_compute_force", "fl_advance", "fl_run", "fl_destroy"):
        assert want in names


def test_library_exports_every_declared_symbol():
    lib = _lib.lib()
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert declared_symbols() <= exported


def test_python_signatures_cover_the_header():
    assert {s for s, _, _ in _lib.SIGNATURES} == declared_symbols()


def test_abi_version_and_struct_size():
    assert _lib.lib().fl_abi_version() == 1
    # 27 input words + 35 derived words + 216 adjacency entries, no padding
    # (every member is a 4-byte float or int, so C and ctypes agree)
    assert C.sizeof(F.FlParams) == 4 * (27 + 35 + 216)


def test_default_params_match_setup_default_params():
    p = F.default_params()
    # fluids4.0/fluid_system.cpp:1987-2008 and 125, 2081-2088
    assert np.float32(p.dt) == np.float32(0.003) and np.float32(p.sim_scale) == np.float32(0.004)
    assert np.float32(p.prest_dens) == np.float32(400.0) and np.float32(p.pintstiff) == np.float32(1.5)
    assert p.grid_density == 2.0 and list(p.bound_max) == [40.0, 60.0, 40.0]
    d = F.derive_params(p)
    assert d.gridSrch == 3 and d.gridAdjCnt == 27


def test_dam_break_grid_is_17_cubed(golden_dir):
    """cell = 0.02 m at sim_scale 0.004 is 4.9999995 world units in FP32, so
    the 80-unit span needs ceil(16.0000016) = 17 cells per axis."""
    p = scenes.dam_break(n=8).params
    assert list(p.gridRes) == [17, 17, 17] and p.gridTotal == 4913
    assert p.gridSrch == 2 and list(p.gridAdj[:8]) == [0, 1, 17, 18, 289, 290, 306, 307]
    assert list(p.gridScanMax) == [15, 15, 15]


@pytest.mark.parametrize("name", ["dam_break_32k", "wave_tank_4m", "kat"])
def test_derivation_matches_golden(golden_dir, name):
    want = json.loads((golden_dir / "params.json").read_text())[name]
    p = F.default_params()
    for k in F.FlParams.INPUTS:
        p.set(**{k: want[k]})
    got = F.derive_params(p).as_dict()
    for k, v in want.items():
        if k in ("poly6kern", "spikykern", "lapkern"):
            # powf: a libm build may round the last place differently
            a, b = np.float32(got[k]), np.float32(v)
            assert abs(int(a.view(np.int32)) - int(b.view(np.int32))) <= 1, k
        else:
            assert np.array_equal(np.asarray(got[k], np.float64), np.asarray(v, np.float64)), k


@pytest.mark.parametrize("gd", [0.5, 0.75, 1.0, 1.2, 2.0, 3.0])
def test_derivation_matches_independent_restatement(gd):
    p = scenes.make_params((-30.0, 0.0, -30.0), (30.0, 60.0, 30.0), grid_density=gd)
    assert PO.compare(p, tol_ulps=0) == []


def test_fatal_search_width_is_an_error_not_an_exit():
    # grid_density 4 -> cell 0.375 h -> gridSrch = floor(2/0.375)+1 = 6 (ok);
    # 5 -> cell 0.3 h -> 7 (fatal upstream, cpp:830-833)
    p = scenes.make_params((-30.0, 0.0, -30.0), (30.0, 60.0, 30.0), grid_density=4.0)
    assert p.gridSrch == 6
    bad = F.default_params()
    bad.set(**scenes.SPH_PARAMS)
    bad.grid_density = 5.0
    with pytest.raises(F.FluidsError) as e:
        F.derive_params(bad)
    assert e.value.code == -3 and "6" in str(e.value)


def test_null_arguments_are_rejected():
    lib = _lib.lib()
    assert lib.fl_params_derive(None) == -1
    assert lib.fl_create(None, 10, None) == -1
    assert b"null" in lib.fl_last_error()
    assert lib.fl_run(None) == -1 and lib.fl_sync(None) == -1
    assert lib.fl_destroy(None) == 0


def test_underived_params_are_rejected():
    p = F.default_params()   # derived block still zero
    h = C.c_void_p()
    assert _lib.lib().fl_create(C.byref(p), 100, C.byref(h)) == -3


def test_product_has_no_cpu_fallback():
    """The product package never imports the oracle and never loads a host
    implementation of the step."""
    pkg = ROOT / "fluids3_gb300"
    for f in pkg.rglob("*.py"):
        text = f.read_text()
        assert "oracle" not in text.replace("oracle/", ""), f"{f} mentions the oracle"
    for f in (pkg / "csrc").iterdir():
        assert "fluids_oracle" not in f.read_text()


def test_oracle_parameter_blocks_equal_the_library_ones():
    """The benchmark's reference arm builds its parameters with the oracle's
    restatement alone (no product code): the blocks must be byte-identical."""
    for n in (60_000, 4_000_000):
        a = scenes.wave_tank(n=n).params
        b = scenes.wave_tank(n=n, derive=PO.derive_flparams).params
        assert bytes(bytearray(a)) == bytes(bytearray(b)), f"wave tank {n}"


def test_noalloc_scan_rejects_bad_arguments_before_any_gpu_work():
    lib = _lib.lib()
    status, counts, offsets = C.c_void_p(0x10000), C.c_void_p(0x20000), C.c_void_p(0x40000)
    assert lib.fl_prefix_sum_noalloc(counts, offsets, 100, 1, None, None) == -1
    assert b"d_status is required" in lib.fl_last_error()
    # ranges [0x20000, 0x20000 + 4n) and [0x20100, ...) overlap for n = 100
    assert lib.fl_prefix_sum_noalloc(counts, C.c_void_p(0x20100), 100, 1, status, None) == -1
    assert b"overlap" in lib.fl_last_error()
    assert lib.fl_prefix_sum_noalloc(counts, offsets, -1, 1, status, None) == -1
    assert lib.fl_prefix_sum_noalloc(None, None, 0, 1, None, None) == 0
    assert lib.fl_test_scan_noalloc_timeout(counts, offsets, 4096, status, 256, None) == -1
    assert b"two tiles" in lib.fl_last_error()
    assert lib.fl_test_scan_noalloc_timeout(counts, offsets, 8192, status, 0, None) == -1
    assert lib.fl_test_scan_timeout(None, 256) == -1


def test_reference_arm_loads_no_product_library():
    """bench.py --impl reference times the reference's CPU path; its scene
    parameters come from the oracle's own derivation, so the product library
    is never loaded in that process (checked in a fresh one)."""
    code = (
        "import sys, runpy\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--n', '12000', '--steps', '1', '--warmup', '0']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('PRODUCT_LOADED' if 'libfluids_gb300' in maps else 'PRODUCT_NOT_LOADED')\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert "PRODUCT_NOT_LOADED" in out.stdout


def header_defines(prefix: str) -> dict[str, int]:
    out = {}
    for h in HEADERS:
        for m in re.finditer(rf"^#define\s+({prefix}[A-Z_0-9]*)\s+\(?(\d+)", h.read_text(), re.M):
            out[m.group(1)] = int(m.group(2))
    return out


def test_python_mode_names_follow_the_header_values():
    """SetNeighbourPasses / NeighbourPasses index system.PASSES by the
    FL_PASSES_* values: the names must sit at those values."""
    from fluids3_gb300 import system
    passes = header_defines("FL_PASSES_")
    assert passes == {"FL_PASSES_PER_POINT": 0, "FL_PASSES_CELL_TASKS": 1, "FL_PASSES_POINT_PAIRS": 2,
                      "FL_PASSES_AUTO": 3}
    names = {"FL_PASSES_PER_POINT": "points", "FL_PASSES_CELL_TASKS": "cells",
             "FL_PASSES_POINT_PAIRS": "pairs", "FL_PASSES_AUTO": "auto"}
    for define, value in passes.items():
        assert system.PASSES[value] == names[define]
    reverse = header_defines("FL_REVERSE_")
    assert reverse["FL_REVERSE_AUTO"] == 0 and reverse["FL_REVERSE_WALK"] == 1
    assert reverse["FL_REVERSE_TRANSPOSE"] == 2
