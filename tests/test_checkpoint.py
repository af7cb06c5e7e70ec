"""Checkpoint text (pps_checkpoint_format / _parse) in the reference's format
and with its validation rules (main.c:304-372, pps/app.c:1301-1352).  CPU only."""
from __future__ import annotations

import pytest


def _job(pps):
    return pps.normalize(pmin=42 * 10**12, pmax=42 * 10**12 + 10**11, kmin=1201, kmax=9999,
                         nmin=2000000, nmax=3000000)


def test_format_is_the_references(pps):
    jp = _job(pps)
    c = pps.Checkpoint(jp.pmin, jp.pmin + 123456789, 4242, 0x1234abcd5678ef01, jp.nmin, jp.nmax, 7, 0)
    text = pps.checkpoint_format(c)
    checksum = (c.pmin + c.p + c.count + c.sum) & (2**64 - 1)
    want = (f"pmin={c.pmin},p={c.p},count={c.count},sum=0x{c.sum:016x},checksum=0x{checksum:016x}\n"
            f"nmin={c.nmin},nmax={c.nmax},factor_count={c.factor_count}\n")
    assert text == want
    back = pps.checkpoint_parse(text, jp)
    assert (back.p, back.count, back.sum, back.factor_count) == (c.p, c.count, c.sum, 7)


def test_invalid_checkpoints_are_refused(pps):
    jp = _job(pps)
    good = pps.Checkpoint(jp.pmin, jp.pmin + 1000, 10, 99, jp.nmin, jp.nmax, 0, 0)
    text = pps.checkpoint_format(good)
    bad_sum = text.replace("sum=0x0000000000000063", "sum=0x0000000000000064")
    other_n = text.replace(f"nmax={jp.nmax}", f"nmax={jp.nmax + 1}")
    outside = pps.checkpoint_format(pps.Checkpoint(jp.pmin, jp.pmax, 10, 99, jp.nmin, jp.nmax, 0, 0))
    at_start = pps.checkpoint_format(pps.Checkpoint(jp.pmin, jp.pmin, 0, 0, jp.nmin, jp.nmax, 0, 0))
    for t in (bad_sum, other_n, outside, at_start, "garbage", text.splitlines()[0]):
        with pytest.raises(pps.PPSError) as ei:
            pps.checkpoint_parse(t, jp)
        assert ei.value.code == pps.PPS_ERR_INVALID_PARAM
