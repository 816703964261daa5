"""Checkpoint files (lbm_save_checkpoint / lbm_create_from_checkpoint): the
header is validated before any device is touched, so corrupt or truncated
files are rejected with LBM_ERR_IO on a machine without a GPU, and a valid
header gets as far as the device check."""
import ctypes as C
import struct

import pytest

LBM_ERR_IO = 7
LBM_ERR_NO_DEVICE = 10
MAGIC = b"LBMGB300CKPT\0\0\0\0"
ELEM = {0: 8, 1: 4, 2: 2, 3: 2, 4: 2}  # bytes per population: f64, f32, f16s, bf16s, f16sr


def header(storage=1, n=(6, 5, 4), fma=0, version=1, magic=MAGIC, flag_bytes=None, pop_bytes=None, lid=None):
    """Version 1 has no lid record; version 2 appends (lid mode, moving wall)."""
    cells = (n[0] + 2) * (n[1] + 2) * (n[2] + 2)
    flag_bytes = cells if flag_bytes is None else flag_bytes
    pop_bytes = 19 * cells * ELEM.get(storage, 4) if pop_bytes is None else pop_bytes
    h = struct.pack("<16sIiiiiqiidddddiiiiiiQQ", magic, version, storage, *n, 12, 0, fma, 1.6, 0.05, 0.0, 0.0,
                    0.0, 1, 1, 1, 1, 1, 1, flag_bytes, pop_bytes)
    if lid is not None:
        h += struct.pack("<ii", *lid)
    return h


def test_header_layout():
    # magic, version, storage, size, counter, last_alpha, fma, 5 doubles, 6 faces, 2 sizes
    assert len(header()) == 16 + 4 + 16 + 8 + 8 + 40 + 24 + 16


def _open(lib, path):
    h = C.c_void_p()
    return lib.lbm_create_from_checkpoint(str(path).encode(), 0, C.byref(h)), h


@pytest.mark.parametrize("case", ["missing", "empty", "truncated", "magic", "version", "storage", "size", "huge", "fma",
                                  "flag_bytes", "pop_bytes", "lid_missing", "lid_mode", "lid_moving"])
def test_corrupt_checkpoints_are_rejected(lib, tmp_path, case):
    path = tmp_path / "c.ckpt"
    data = {
        "empty": b"",
        "truncated": header()[:100],
        "magic": header(magic=b"LBMGB300CKPX\0\0\0\0"),
        "version": header(version=3),
        "lid_missing": header(version=2),                      # version 2 without its lid record
        "lid_mode": header(version=2, lid=(2, 0)),
        "lid_moving": header(version=2, lid=(0, 1)),           # only a moving-wall lid moves
        "storage": header(storage=7),
        "size": header(n=(6, 0, 4)),
        "huge": header(n=(2 ** 31 - 2, 1, 1)),  # beyond lbm_create's 2^20 per axis; nx + 2 overflows int32
        "fma": header(fma=2),
        "flag_bytes": header(flag_bytes=10),
        "pop_bytes": header(storage=2, pop_bytes=19 * 8 * 7 * 6 * 4),
    }.get(case)
    if data is not None:
        path.write_bytes(data)
    rc, h = _open(lib, path)
    assert rc == LBM_ERR_IO and not h.value, case
    assert lib.lbm_status_string(rc)


def test_valid_header_reaches_the_device_check(lib, tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible: the GPU tests cover resuming")
    for storage in (0, 1, 2, 3, 4):
        path = tmp_path / f"ok{storage}.ckpt"
        path.write_bytes(header(storage=storage, fma=1 if storage == 0 else 0))
        rc, h = _open(lib, path)
        assert rc == LBM_ERR_NO_DEVICE and not h.value, storage
    for lid in ((0, 0), (1, 0), (1, 1)):  # version 2: injection lid, wall at rest, moving wall
        path = tmp_path / f"v2_{lid[0]}{lid[1]}.ckpt"
        path.write_bytes(header(version=2, lid=lid))
        rc, h = _open(lib, path)
        assert rc == LBM_ERR_NO_DEVICE and not h.value, lid
