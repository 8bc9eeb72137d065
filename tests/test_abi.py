"""C-ABI checks that need no GPU: the library loads, exports every entry point
include/strouhal_c.h declares, reports a missing device as an error status, and
its host utilities (SHA-256, solid-fraction generators) are correct."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "strouhal_c.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(stro_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def sg():
    import strouhal_gb300

    if not os.path.exists(strouhal_gb300.LIB_PATH):
        from strouhal_gb300 import build

        build.build()
    strouhal_gb300.lib()
    return strouhal_gb300


def test_every_declared_symbol_is_exported(sg):
    decl = _declared()
    assert len(decl) >= 35
    out = subprocess.run(["nm", "-D", "--defined-only", sg.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(stro_\w+)\b", out))
    missing = [d for d in decl if d not in exported]
    assert not missing, missing
    L = sg.lib()
    for d in decl:
        assert hasattr(L, d)


def test_abi_version(sg):
    assert sg.lib().stro_abi_version() == 1


def test_no_device_is_an_error_status(sg):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sg.StrouhalError) as ei:
        sg.GPU(0)
    assert ei.value.code == 2


def test_sha256_matches_hashlib(sg):
    rng = np.random.default_rng(3)
    for n in (0, 1, 55, 56, 63, 64, 65, 119, 120, 1000, 1 << 20):
        b = rng.bytes(n)
        assert sg.sha256Hex(b) == hashlib.sha256(b).hexdigest(), n


def _disk_py(nx, ny, cx, cy, r):
    """CaseSetups.swift:6-25 restated in numpy."""
    eps = np.zeros((ny, nx), np.float32)
    sub = 16
    o = (np.arange(sub) + 0.5) / sub - 0.5
    for y in range(max(0, int(cy - r) - 2), min(ny - 1, int(cy + r) + 2) + 1):
        for x in range(max(0, int(cx - r) - 2), min(nx - 1, int(cx + r) + 2) + 1):
            px = x + o[None, :]
            py = y + o[:, None]
            inside = np.count_nonzero((px - cx) ** 2 + (py - cy) ** 2 <= r * r)
            eps[y, x] = np.float32(inside) / np.float32(sub * sub)
    return eps.reshape(-1)


def test_disk_solid_fractions(sg):
    a = sg.diskSolidFractions(60, 40, 20.5, 19.5, 9.0)
    assert np.array_equal(a, _disk_py(60, 40, 20.5, 19.5, 9.0))
    assert abs(a.sum() - np.pi * 81) < 0.5


def test_sphere_solid_fractions(sg):
    a = sg.sphereSolidFractions(24, 20, 22, 11.5, 10.0, 10.7, 6.0, sub=8).reshape(22, 20, 24)
    assert abs(a.sum() - 4.0 / 3.0 * np.pi * 216) < 2.0
    # one cell by direct sampling
    z, y, x = 10, 10, 14
    o = (np.arange(8) + 0.5) / 8 - 0.5
    P = np.stack(np.meshgrid(x + o, y + o, z + o, indexing="ij"), -1)
    inside = np.count_nonzero(((P - [11.5, 10.0, 10.7]) ** 2).sum(-1) <= 36.0)
    assert a[z, y, x] == np.float32(inside) / np.float32(512)


def test_plain_c_client_compiles_links_and_runs(sg, tmp_path):
    """The header is C99 (what a cgo, Swift or ctypes binding reads) and the
    library links from C; on a machine without a GPU the client sees
    STRO_ERR_NO_DEVICE with a message."""
    exe = str(tmp_path / "c_client")
    libdir = os.path.dirname(sg.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c_client.c"),
                    "-L", libdir, "-lstrouhal_gb300", "-Wl,-rpath," + libdir, "-o", exe],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    import torch

    if not torch.cuda.is_available():
        assert r.stdout.startswith("no-device ")
    else:
        assert r.stdout.startswith("digest ")
