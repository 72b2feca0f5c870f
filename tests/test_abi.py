"""The C-ABI library: it loads, exports every symbol that include/*.h
declares, and validates arguments before touching the GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"^MHD_API\s+[^;(]*?\b(\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol(mhd):
    L = mhd.lib()
    names = declared_symbols()
    for ref_name in ("fluidx", "advectbyzx", "transpose12", "transpose13", "calcfl", "copy_matrix"):
        assert ref_name in names
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_reference_signatures_in_header():
    """The drop-in prototypes are those of C/spu_function.h:1-15."""
    text = (ROOT / "include" / "mhd_gb300.h").read_text()
    flat = re.sub(r"\s+", " ", text)
    for proto in [
        "void fluidx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u, float *update_b, int iter)",
        "void copy_matrix(float *u, float *b, int *nx, int *ny, int *nz, float *update_u, float *update_b)",
        "void advectbyzx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u, float *update_b)",
        "void transpose12(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz, int iter)",
        "void transpose13(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz)",
        "float calcfl(float *u, float *b, int *nx, int *ny, int *nz)",
    ]:
        assert proto in flat, proto


def test_error_strings_and_argument_checks(mhd):
    L = mhd.lib()
    assert L.mhd_error_string(0) == b"ok"
    assert L.mhd_error_string(1) == b"bad argument"
    h = C.c_void_p()
    assert L.mhd_create(C.byref(h), 0, 4, 4, 0) == 1  # rejected before any CUDA call
    assert L.mhd_create(None, 4, 4, 4, 0) == 1
    n = C.c_int(4)
    L.fluidx(None, None, C.byref(n), C.byref(n), C.byref(n), C.byref(C.c_float(0.1)), None, None, 0)
    assert L.mhd_last_error() == 1
    L.calcfl(None, None, None, None, None)
    assert L.mhd_last_error() == 1
    # batched boxes: edges outside 1..512 and empty batches, before any CUDA call
    for sizes in ([32, 0], [513], [-4]):
        arr = (C.c_int * len(sizes))(*sizes)
        assert L.mhd_batch_create(C.byref(h), len(sizes), arr, 0) == 1
    assert L.mhd_batch_create(C.byref(h), 0, (C.c_int * 1)(32), 0) == 1
    assert L.mhd_batch_step(None, 1, 0.7) == 1
    assert L.mhd_batch_set_box(None, 0, None, None, 0) == 1


def test_batch_config_table(mhd):
    cfg = mhd.batch_config(256, seed=0)
    assert cfg == mhd.batch_config(256, seed=0)
    assert {x["n"] for x in cfg} == set(mhd.BATCH_EDGES)
    assert all(0.1 <= x["beta"] <= 10 and 0.2 <= x["mach"] <= 1.0 for x in cfg)
    assert len({x["seed"] for x in cfg}) == 256
    # p and v follow beta and Mach (rho = 1, gamma = 5/3, <B^2> = 1/(4 pi))
    box = dict(n=16, seed=4, beta=2.0, mach=0.5)
    u, b = mhd.init_batch_box(box)
    U, B = u.reshape(-1, 5).astype(np.float64), b.reshape(-1, 3).astype(np.float64)
    ekin = 0.5 * (U[:, 1:4] ** 2).sum(1) / U[:, 0]
    B4 = B.reshape(16, 16, 16, 3)  # (k, j, i, component); B_c is the face average
    bc = 0.5 * (B4 + np.stack([np.roll(B4[..., c], -1, axis=2 - c) for c in range(3)], axis=-1))
    p = (U[:, 4] - ekin - 0.5 * (bc.reshape(-1, 3) ** 2).sum(1)) * (2.0 / 3.0)
    assert np.allclose(p, 2.0 / (8 * np.pi), rtol=1e-4)
    v_rms = np.sqrt(((U[:, 1:4] / U[:, :1]) ** 2).sum(1).mean())
    assert abs(v_rms / np.sqrt(5.0 / 3.0 * 2.0 / (8 * np.pi)) - 0.5) < 0.02


def test_no_cpu_fallback_in_product():
    """The product never loads the oracle: no reference to oracle/ in the package."""
    pkg = ROOT / "heterogeneous_mhd_gb300"
    for p in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")) + list(pkg.rglob("*.c")):
        text = p.read_text()
        assert "liboracle" not in text and "orc_" not in text and "oracle/" not in text, p
