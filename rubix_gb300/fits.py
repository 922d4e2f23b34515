"""Minimal FITS reader and writer (image HDUs), for the cube output and the FITS SSP
templates on either side of the particle -> cube path.

rubix uses astropy.io.fits (core/fits.py:13-102, spectra/ssp/grid.py:518-581), which is
not a dependency here.  This module implements the parts of the FITS standard (version
4.0) those calls use: a primary HDU and IMAGE extensions, fixed-format 80-character
header cards (logical, integer, floating-point and string values with comments),
2880-byte blocks, big-endian data with BITPIX 8/16/32/64/-32/-64 and BSCALE/BZERO on
read, gzip-compressed files on read.
"""

from __future__ import annotations

import gzip
from dataclasses import dataclass, field
from typing import Any, Iterable, List, Optional, Sequence, Tuple

import numpy as np

__all__ = ["HDU", "Header", "read_fits", "write_fits", "format_card", "BLOCK"]

BLOCK = 2880
_BITPIX_DTYPE = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


class Header:
    """Ordered FITS header: (key, value, comment) cards with dict-style access."""

    def __init__(self, cards: Iterable[Tuple[str, Any, str]] = ()):
        self.cards: List[List[Any]] = []
        for k, v, *c in cards:
            self[k] = (v, c[0] if c else "")

    def __setitem__(self, key: str, value) -> None:
        comment = ""
        if isinstance(value, tuple):
            value, comment = value
        key = key.upper()
        for card in self.cards:
            if card[0] == key:
                card[1], card[2] = value, comment or card[2]
                return
        self.cards.append([key, value, comment])

    def __getitem__(self, key: str):
        key = key.upper()
        for k, v, _ in self.cards:
            if k == key:
                return v
        raise KeyError(key)

    def get(self, key: str, default=None):
        try:
            return self[key]
        except KeyError:
            return default

    def __contains__(self, key: str) -> bool:
        return any(k == key.upper() for k, _, _ in self.cards)

    def keys(self):
        return [k for k, _, _ in self.cards]


@dataclass
class HDU:
    header: Header
    data: Optional[np.ndarray] = None  # native-endian array, shape (NAXISn, ..., NAXIS1)
    raw: Optional[bytes] = field(default=None, repr=False)


def _format_value(v) -> str:
    if isinstance(v, (bool, np.bool_)):
        return f"{'T' if v else 'F':>20}"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):>20d}"
    if isinstance(v, (float, np.floating)):
        s = repr(float(v)).upper()
        mant, e, exp = s.partition("E")
        if "." not in mant and mant.lstrip("-").isdigit():
            s = mant + ".0" + e + exp
        if len(s) > 20:
            s = f"{float(v):.16E}"
        return f"{s:>20}"
    s = str(v).replace("'", "''")
    return f"'{s:<8}'"


def format_card(key: str, value=None, comment: str = "") -> str:
    """One 80-character header card in the fixed format: keyword in columns 1-8,
    '= ' in 9-10, numbers and logicals right-justified to column 30, strings quoted
    from column 11 (at least 8 characters between the quotes)."""
    key = key.upper()
    if len(key) > 8:
        raise ValueError(f"FITS keyword {key!r} longer than 8 characters")
    if key in ("COMMENT", "HISTORY", "") or value is None:
        text = (f"{key:<8}" + ("  " + str(comment) if comment else ""))[:80]
    else:
        text = f"{key:<8}= {_format_value(value)}"
        if len(text) > 80:
            raise ValueError(f"FITS value of {key} does not fit one card")
        if comment:
            text = (text + f" / {comment}")[:80]
    return f"{text:<80}"


def _header_bytes(cards: Sequence[Tuple[str, Any, str]]) -> bytes:
    text = "".join(format_card(k, v, c) for k, v, c in cards) + f"{'END':<80}"
    raw = text.encode("ascii")
    return raw + b" " * ((-len(raw)) % BLOCK)


def _image_cards(data_shape: Tuple[int, ...], bitpix: int, primary: bool,
                 extend: bool = False) -> List[Tuple[str, Any, str]]:
    cards = [("SIMPLE", True, "conforms to FITS standard")] if primary else \
        [("XTENSION", "IMAGE", "Image extension")]
    cards.append(("BITPIX", bitpix, "array data type"))
    cards.append(("NAXIS", len(data_shape), "number of array dimensions"))
    for i, n in enumerate(reversed(data_shape)):
        cards.append((f"NAXIS{i + 1}", int(n), ""))
    if primary:
        if extend:
            cards.append(("EXTEND", True, ""))
    else:
        cards.append(("PCOUNT", 0, "number of parameters"))
        cards.append(("GCOUNT", 1, "number of groups"))
    return cards


_RESERVED = {"SIMPLE", "XTENSION", "BITPIX", "NAXIS", "EXTEND", "PCOUNT", "GCOUNT", "END"}


def write_fits(path: str, hdus: Sequence[HDU]) -> None:
    """Write HDUs (the first is the primary) to ``path``.  An HDU's data may be given
    as an array (written big-endian with the matching BITPIX) or as ``raw`` bytes that
    are already big-endian, with ``header["BITPIX"]`` and ``NAXISn`` describing them."""
    with open(path, "wb") as f:
        for i, h in enumerate(hdus):
            primary = i == 0
            if h.raw is not None:
                shape = tuple(int(h.header[f"NAXIS{k}"])
                              for k in range(int(h.header["NAXIS"]), 0, -1))
                bitpix = int(h.header["BITPIX"])
                payload = h.raw
            elif h.data is not None:
                arr = np.asarray(h.data)
                bitpix = {np.dtype(v).newbyteorder("="): k
                          for k, v in _BITPIX_DTYPE.items()}.get(arr.dtype.newbyteorder("="))
                if bitpix is None:
                    raise ValueError(f"no FITS BITPIX for dtype {arr.dtype}")
                shape = arr.shape
                payload = np.ascontiguousarray(arr, dtype=_BITPIX_DTYPE[bitpix]).tobytes()
            else:
                shape, bitpix, payload = (), 8, b""
            cards = _image_cards(shape, bitpix, primary, extend=primary and len(hdus) > 1)
            for k, v, c in h.header.cards:
                if k in _RESERVED or (k.startswith("NAXIS") and k[5:].isdigit()):
                    continue
                cards.append((k, v, c))
            f.write(_header_bytes(cards))
            if payload:
                f.write(payload)
                f.write(b"\0" * ((-len(payload)) % BLOCK))


def _parse_value(text: str):
    t = text.strip()
    if not t:
        return None, ""
    if t.startswith("'"):
        # quoted string with '' escapes, then an optional comment
        i, out = 1, []
        while i < len(t):
            if t[i] == "'":
                if i + 1 < len(t) and t[i + 1] == "'":
                    out.append("'")
                    i += 2
                    continue
                break
            out.append(t[i])
            i += 1
        rest = t[i + 1:]
        comment = rest.split("/", 1)[1].strip() if "/" in rest else ""
        return "".join(out).rstrip(), comment
    val, _, comment = t.partition("/")
    val = val.strip()
    comment = comment.strip()
    if val == "T":
        return True, comment
    if val == "F":
        return False, comment
    try:
        return int(val), comment
    except ValueError:
        pass
    try:
        return float(val.replace("D", "E")), comment
    except ValueError:
        return val, comment


def _read_header(buf: bytes, pos: int) -> Tuple[Header, int]:
    hdr = Header()
    while True:
        if pos + BLOCK > len(buf):
            raise ValueError("truncated FITS header")
        block = buf[pos:pos + BLOCK].decode("ascii", errors="replace")
        pos += BLOCK
        for i in range(0, BLOCK, 80):
            card = block[i:i + 80]
            key = card[:8].strip()
            if key == "END":
                return hdr, pos
            if card[8:10] == "= ":
                v, c = _parse_value(card[10:])
                hdr.cards.append([key, v, c])
            elif key:
                hdr.cards.append([key, None, card[8:].strip()])


def read_fits(path_or_bytes) -> List[HDU]:
    """Every HDU of a FITS file (gzip-compressed files are read too): headers and data
    as native-endian arrays of shape (NAXISn, ..., NAXIS1), BSCALE/BZERO applied."""
    if isinstance(path_or_bytes, (bytes, bytearray)):
        buf = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            buf = f.read()
    if buf[:2] == b"\x1f\x8b":
        buf = gzip.decompress(buf)
    hdus, pos = [], 0
    while pos + BLOCK <= len(buf):
        hdr, pos = _read_header(buf, pos)
        naxis = int(hdr.get("NAXIS", 0))
        shape = tuple(int(hdr[f"NAXIS{k}"]) for k in range(naxis, 0, -1))
        bitpix = int(hdr["BITPIX"])
        count = int(np.prod(shape)) if naxis else 0
        nbytes = abs(bitpix) // 8 * int(hdr.get("GCOUNT", 1)) * (int(hdr.get("PCOUNT", 0)) + count)
        data = None
        if count:
            raw = np.frombuffer(buf, dtype=_BITPIX_DTYPE[bitpix], count=count, offset=pos)
            data = raw.astype(raw.dtype.newbyteorder("=")).reshape(shape)
            bscale, bzero = hdr.get("BSCALE", 1), hdr.get("BZERO", 0)
            if bscale != 1 or bzero != 0:
                data = data * np.float64(bscale) + np.float64(bzero)
        hdus.append(HDU(hdr, data))
        pos += nbytes + ((-nbytes) % BLOCK)
    return hdus
