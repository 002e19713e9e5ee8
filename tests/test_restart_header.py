"""Restart-file header checks, host only (emoo_restart_info; emoo_read_restart
runs the same checks before it changes a handle).

The files are written here byte by byte in the library's layout: a fixed
header (RestartHeader in csrc/io.cpp), the history rows, the fields and the
particle arrays. A well-formed file is accepted; a short file, a negative or
inconsistent species count, a huge history-row count, an unknown flag value
or a gamma array the writer never stores are refused with EMOO_ERR_INPUT.
"""
import ctypes as C
import struct

import pytest

from apc_524_project_gb300 import abi

NSPEC = 32
FP64, MIXED = 0, 1


def header(precision=MIXED, n=(2, 3, 4), nspec=2, counts=(3, 2), has_ids=1, has_gam=0, has_g0=0,
           first_push=0, nhist=1, np_=None, flags=None):
    cnt = list(counts) + [0] * (NSPEC - len(counts))
    np_ = sum(cnt) if np_ is None else np_
    f = dict(bswap=0, rho_stale=0, first_push=first_push, has_ids=has_ids, has_gam=has_gam, has_g0=has_g0,
             dead_pending=0)
    f.update(flags or {})
    h = b"EMOORST1"
    h += struct.pack("<6i", 1, precision, *n, nspec)
    h += struct.pack("<8i", f["bswap"], f["rho_stale"], f["first_push"], f["has_ids"], f["has_gam"], f["has_g0"],
                     f["dead_pending"], 0)
    h += struct.pack("<33q", np_, *cnt)
    h += struct.pack("<3d", 1.5, 0.5, 0.5)
    h += struct.pack("<3q", 3, 10, nhist)
    assert len(h) == 376
    return h, np_


def body(precision, n, np_, has_ids, has_gam, has_g0, nhist):
    npts = (n[0] + 3) * (n[1] + 3) * (n[2] + 3)
    if precision == FP64:
        field = 13 * 8 * npts
        part = 48 + (8 if has_gam else 0)
    else:
        field = 9 * 4 * npts + 4 * 8 * npts
        part = 28 + (4 if has_g0 else 0)
    part += 8 if has_ids else 0
    return bytes(nhist * 64 + field + np_ * part)


def write(path, **kw):
    h, np_ = header(**kw)
    args = dict(precision=kw.get("precision", MIXED), n=kw.get("n", (2, 3, 4)), np_=np_,
                has_ids=kw.get("has_ids", 1), has_gam=kw.get("has_gam", 0), has_g0=kw.get("has_g0", 0),
                nhist=kw.get("nhist", 1))
    if args["nhist"] > 1000:
        args["nhist"] = 1
    data = h + body(**args)
    path.write_bytes(data)
    return data


def info(path):
    d = abi.RestartDesc()
    rc = abi.lib().emoo_restart_info(str(path).encode(), C.byref(d))
    return rc, d


def test_well_formed_files_are_read(tmp_path):
    p = tmp_path / "ok.rst"
    write(p)
    rc, d = info(p)
    assert rc == abi.OK
    assert (d.precision, list(d.n), d.nspec, d.has_ids, d.np) == (MIXED, [2, 3, 4], 2, 1, 5)
    assert list(d.count[:3]) == [3, 2, 0] and d.step_index == 3 and d.nhist_rows == 1 and d.t == 1.5
    write(p, precision=FP64, has_gam=1, has_ids=0, nhist=0)
    assert info(p)[0] == abi.OK
    write(p, has_g0=1, first_push=1)
    assert info(p)[0] == abi.OK
    write(p, counts=(0, 0), has_ids=1)  # an empty store
    assert info(p)[0] == abi.OK


def test_truncated_and_padded_files_are_refused(tmp_path):
    p = tmp_path / "t.rst"
    data = write(p)
    for cut in (10, 376, len(data) - 1):
        p.write_bytes(data[:cut])
        assert info(p)[0] == abi.ERR_INPUT, cut
    p.write_bytes(data + b"\0")
    assert info(p)[0] == abi.ERR_INPUT


@pytest.mark.parametrize("kw", [
    dict(counts=(3, -1)),                 # negative count
    dict(counts=(3, 2), np_=4),           # counts do not sum to np
    dict(counts=(3, 2, 1), nspec=2),      # a count past nspec
    dict(nhist=1 << 50),                  # history rows beyond any file
    dict(flags=dict(bswap=2)),            # flags are 0 or 1
    dict(precision=FP64, has_gam=0),      # FP64 particles always carry gamma
    dict(has_gam=1),                      # the mixed form has no FP64 gamma
    dict(has_g0=1, first_push=0),         # the loaded gamma exists only before the first push
    dict(precision=7),
    dict(n=(0, 3, 4)),
])
def test_inconsistent_headers_are_refused(tmp_path, kw):
    p = tmp_path / "bad.rst"
    write(p, **kw)
    assert info(p)[0] == abi.ERR_INPUT


def test_missing_file_and_null_arguments(tmp_path):
    assert info(tmp_path / "none.rst")[0] == abi.ERR_INPUT
    assert abi.lib().emoo_restart_info(None, None) == abi.ERR_ARG
