"""Minimal FITS primary-HDU reader / writer (no astropy needed).

Covers what FitsImage needs (pymoresane/main.py:618-646,681-724): a primary
HDU with BITPIX 8/16/32/64/-32/-64, NAXIS 1-4, optional BSCALE/BZERO; the
header is kept as an ordered list of 80-character cards so that a written
model / residual carries the input image's keywords.
"""
import numpy as np

BLOCK = 2880
_DTYPES = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}
_STRUCTURAL = ("SIMPLE", "BITPIX", "NAXIS", "EXTEND", "END", "BSCALE", "BZERO")


class Header:
    """Ordered FITS cards with dict-style access to keyword values."""

    def __init__(self, cards):
        self.cards = list(cards)

    @staticmethod
    def _parse_value(text):
        v = text.split("/")[0].strip() if not text.strip().startswith("'") else text.strip()
        if v.startswith("'"):
            end = v.find("'", 1)
            return v[1:end].rstrip()
        if v in ("T", "F"):
            return v == "T"
        try:
            return int(v)
        except ValueError:
            try:
                return float(v.replace("D", "E"))
            except ValueError:
                return v

    def keys(self):
        return [c[:8].strip() for c in self.cards]

    def __contains__(self, key):
        return key in self.keys()

    def __getitem__(self, key):
        for c in self.cards:
            if c[:8].strip() == key and c[8:10] == "= ":
                return self._parse_value(c[10:])
        raise KeyError(key)

    def get(self, key, default=None):
        try:
            return self[key]
        except KeyError:
            return default

    def set(self, key, value):
        if isinstance(value, bool):
            text = "T" if value else "F"
        elif isinstance(value, str):
            text = "'" + value.ljust(8) + "'"
        elif isinstance(value, (int, np.integer)):
            text = str(int(value))
        else:
            text = repr(float(value)).upper()
        card = f"{key:<8}= {text:>20}"[:80].ljust(80)
        for i, c in enumerate(self.cards):
            if c[:8].strip() == key:
                self.cards[i] = card
                return
        self.cards.append(card)


def read(path):
    """Return (data ndarray in FITS axis order reversed, i.e. C order, Header)."""
    with open(path, "rb") as fh:
        raw = fh.read()
    cards, off = [], 0
    while True:
        block = raw[off:off + BLOCK].decode("ascii")
        off += BLOCK
        done = False
        for i in range(0, BLOCK, 80):
            card = block[i:i + 80]
            if card[:8].strip() == "END":
                done = True
                break
            if card.strip():
                cards.append(card)
        if done:
            break
    hdr = Header(cards)
    naxis = hdr["NAXIS"]
    shape = tuple(hdr[f"NAXIS{i}"] for i in range(naxis, 0, -1))
    dtype = np.dtype(_DTYPES[hdr["BITPIX"]])
    count = int(np.prod(shape)) if shape else 0
    data = np.frombuffer(raw[off:off + count * dtype.itemsize], dtype=dtype).reshape(shape)
    data = data.astype(dtype.newbyteorder("="))
    bscale, bzero = hdr.get("BSCALE", 1), hdr.get("BZERO", 0)
    if bscale != 1 or bzero != 0:
        data = data * bscale + bzero
    return data, hdr


def write(path, data, header=None):
    """Write a float32 primary HDU (BITPIX -32), copying non-structural cards of ``header``."""
    data = np.ascontiguousarray(data, dtype=">f4")
    cards = ["SIMPLE  =                    T".ljust(80), "BITPIX  =                  -32".ljust(80),
             f"NAXIS   = {data.ndim:>20}".ljust(80)]
    for i, n in enumerate(reversed(data.shape)):
        cards.append(f"NAXIS{i + 1:<3}= {n:>20}".ljust(80))
    if header is not None:
        for c in header.cards:
            key = c[:8].strip()
            if key.startswith(_STRUCTURAL) or (key.startswith("NAXIS") and key[5:].isdigit()):
                continue
            cards.append(c.ljust(80)[:80])
    cards.append("END".ljust(80))
    head = "".join(cards)
    head += " " * ((-len(head)) % BLOCK)
    body = data.tobytes()
    body += b"\0" * ((-len(body)) % BLOCK)
    with open(path, "wb") as fh:
        fh.write(head.encode("ascii"))
        fh.write(body)
