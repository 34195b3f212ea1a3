"""Futhark value files: the text and binary data formats.

The reference feeds its programs with value files: ``futhark bench`` reads the
datasets named in each program's header (``forwardprojection.fut:1-14``,
``backprojection_sparse.fut:1-12``: ``-- input@data/fpinputf32rad512``), and
the compiled executables read their arguments from standard input in the same
format.  ``data/fpinputf32rad512`` holds the five arguments of
``forwardprojection.main`` as text: ``[0.785...f32, ...] -362.0f32 1.0f32
725i32 [0.0f32, ...]``.

This module reads and writes both encodings of Futhark's published data
format so those files can drive the drop-in classes:

* text: scalars carry a type suffix (``1.5f32``, ``725i32``; an unsuffixed
  integer is ``i32`` and an unsuffixed decimal ``f64``), ``true``/``false``,
  ``f32.nan``/``f32.inf``/``-f32.inf``; arrays are nested ``[...]`` lists;
  ``empty([0][3]f32)`` is an empty array of a given shape; ``--`` starts a
  comment; values are separated by white space.
* binary: ``b``, version byte 2, rank (one signed byte), the element type as
  four ASCII characters right-aligned with spaces (``" f32"``, ``"  i8"``,
  ``"bool"``), ``rank`` little-endian int64 dimensions, then the elements
  little-endian (``bool`` one byte each).  Text and binary values may be mixed
  in one stream.

Values come back as numpy scalars (0-d) or numpy arrays of the value's type.
"""
from __future__ import annotations

import io
import re
import struct
import sys
from typing import BinaryIO, Iterable, List, Sequence, Union

import numpy as np

__all__ = ["FormatError", "read_values", "read_file", "write_text", "write_binary", "format_value", "TYPES"]

# Futhark primitive type name -> numpy dtype
TYPES = {
    "i8": np.int8, "i16": np.int16, "i32": np.int32, "i64": np.int64,
    "u8": np.uint8, "u16": np.uint16, "u32": np.uint32, "u64": np.uint64,
    "f16": np.float16, "f32": np.float32, "f64": np.float64, "bool": np.bool_,
}
_NAME_OF = {np.dtype(v): k for k, v in TYPES.items()}

_NUM = re.compile(
    r"""(?P<sign>-)?
        (?:(?P<special>(?P<sty>f16|f32|f64)\.(?P<sval>nan|inf))
          |(?P<hex>0[xX][0-9a-fA-F_]+)
          |(?P<bin>0[bB][01_]+)
          |(?P<dec>(?:[0-9][0-9_]*(?:\.[0-9_]*)?|\.[0-9][0-9_]*)(?:[eE][+-]?[0-9]+)?))
        (?P<suffix>i8|i16|i32|i64|u8|u16|u32|u64|f16|f32|f64)?""",
    re.VERBOSE,
)
_WS = re.compile(r"(?:\s+|--[^\n]*)*")
_EMPTY = re.compile(r"empty\(\s*((?:\[\s*\d+\s*\]\s*)*)(i8|i16|i32|i64|u8|u16|u32|u64|f16|f32|f64|bool)\s*\)")


class FormatError(ValueError):
    """A malformed value file."""


def _scalar(m: re.Match) -> np.generic:
    neg = m.group("sign") is not None
    suf = m.group("suffix")
    if m.group("special"):
        if suf:
            raise FormatError(f"type suffix after {m.group('special')}")
        dt = TYPES[m.group("sty")]
        v = np.inf if m.group("sval") == "inf" else np.nan
        return dt(-v if neg else v)
    if m.group("hex") or m.group("bin"):
        txt = (m.group("hex") or m.group("bin")).replace("_", "")
        iv = int(txt, 0)
        iv = -iv if neg else iv
        dt = TYPES[suf or "i32"]
        if np.issubdtype(dt, np.floating):
            return dt(iv)
        return _int(dt, iv)
    txt = m.group("dec").replace("_", "")
    is_float = any(c in txt for c in ".eE")
    if suf is None:
        suf = "f64" if is_float else "i32"
    dt = TYPES[suf]
    if np.issubdtype(dt, np.floating):
        v = float(txt)
        return dt(-v if neg else v)
    if is_float:
        raise FormatError(f"decimal literal {txt} with integer suffix {suf}")
    iv = int(txt)
    return _int(dt, -iv if neg else iv)


def _int(dt, iv: int) -> np.generic:
    info = np.iinfo(dt)
    if not info.min <= iv <= info.max:
        raise FormatError(f"{iv} out of range for {_NAME_OF[np.dtype(dt)]}")
    return dt(iv)


class _TextParser:
    def __init__(self, text: str, pos: int = 0):
        self.s = text
        self.p = pos

    def ws(self) -> None:
        self.p = _WS.match(self.s, self.p).end()

    def at_end(self) -> bool:
        self.ws()
        return self.p >= len(self.s)

    def value(self):
        self.ws()
        s, p = self.s, self.p
        if s.startswith("[", p):
            return self.array()
        if s.startswith("empty", p):
            m = _EMPTY.match(s, p)
            if not m:
                raise FormatError(f"bad empty() at offset {p}")
            dims = [int(d) for d in re.findall(r"\d+", m.group(1))]
            if not dims or 0 not in dims:
                raise FormatError(f"empty() needs a zero dimension at offset {p}")
            self.p = m.end()
            return np.zeros(dims, dtype=TYPES[m.group(2)])
        for word, val in (("true", True), ("false", False)):
            if s.startswith(word, p):
                self.p = p + len(word)
                return np.bool_(val)
        m = _NUM.match(s, p)
        if not m or m.end() == p:
            raise FormatError(f"cannot parse a value at offset {p}: {s[p:p + 20]!r}")
        self.p = m.end()
        return _scalar(m)

    def array(self) -> np.ndarray:
        s = self.s
        start = self.p
        # Fast path: a flat array of numeric literals sharing one suffix.
        end = s.find("]", start + 1)
        inner = s[start + 1:end] if end > 0 else ""
        if end > 0 and "[" not in inner and "-- " not in inner and "--" not in inner:
            arr = self._flat(inner)
            if arr is not None:
                self.p = end + 1
                return arr
        self.p += 1
        elems = []
        self.ws()
        if s.startswith("]", self.p):
            raise FormatError(f"empty array literal at offset {start}: write empty([0]t)")
        while True:
            elems.append(self.value())
            self.ws()
            if s.startswith(",", self.p):
                self.p += 1
                continue
            if s.startswith("]", self.p):
                self.p += 1
                break
            raise FormatError(f"expected ',' or ']' at offset {self.p}")
        return _stack(elems, start)

    @staticmethod
    def _flat(inner: str):
        toks = [t.strip() for t in inner.split(",")]
        if not toks or any(not t for t in toks):
            return None
        m = re.search(r"(i8|i16|i32|i64|u8|u16|u32|u64|f16|f32|f64)$", toks[0])
        suf = m.group(1) if m else None
        if suf is None or not all(t.endswith(suf) for t in toks):
            return None
        body = [t[: -len(suf)].replace("_", "") for t in toks]
        dt = TYPES[suf]
        if np.issubdtype(dt, np.floating):
            if any(("." in b and b.endswith(".")) for b in body):
                body = [b + "0" if b.endswith(".") else b for b in body]
            if any(re.search(r"[a-zA-Z]", b.replace("e", "").replace("E", "")) for b in body):
                return None
            return np.array([float(b) for b in body], dtype=np.float64).astype(dt)
        if any(not re.fullmatch(r"-?[0-9]+", b) for b in body):
            return None
        vals = [int(b) for b in body]
        info = np.iinfo(dt)
        if min(vals) < info.min or max(vals) > info.max:
            raise FormatError(f"literal out of range for {suf}")
        return np.array(vals, dtype=dt)


def _stack(elems: list, offset: int) -> np.ndarray:
    first = elems[0]
    shape0 = np.shape(first)
    dt0 = np.asarray(first).dtype
    for e in elems[1:]:
        if np.shape(e) != shape0:
            raise FormatError(f"irregular array at offset {offset}")
        if np.asarray(e).dtype != dt0:
            raise FormatError(f"array elements of different types at offset {offset}")
    return np.stack([np.asarray(e) for e in elems]).astype(dt0, copy=False)


def _binary_value(buf: bytes, p: int):
    if len(buf) < p + 7 or buf[p] != ord("b"):
        raise FormatError(f"not a binary value at offset {p}")
    version = buf[p + 1]
    if version != 2:
        raise FormatError(f"binary format version {version} (expected 2)")
    rank = struct.unpack_from("<b", buf, p + 2)[0]
    tname = buf[p + 3:p + 7].decode("ascii").strip()
    if tname not in TYPES or rank < 0:
        raise FormatError(f"bad binary header at offset {p}: rank {rank}, type {tname!r}")
    p += 7
    dims = list(struct.unpack_from(f"<{rank}q", buf, p)) if rank else []
    p += 8 * rank
    dt = np.dtype(TYPES[tname]).newbyteorder("<")
    count = int(np.prod(dims)) if rank else 1
    nbytes = count * dt.itemsize
    if len(buf) < p + nbytes:
        raise FormatError("truncated binary value")
    arr = np.frombuffer(buf, dtype=dt, count=count, offset=p).astype(dt.newbyteorder("="))
    p += nbytes
    if rank == 0:
        return arr[0], p
    return arr.reshape(dims), p


def read_values(data: Union[bytes, str]) -> List[Union[np.generic, np.ndarray]]:
    """All values of a text or binary (or mixed) Futhark value stream."""
    buf = data.encode("latin-1") if isinstance(data, str) else bytes(data)
    out = []
    p = 0
    ws = re.compile(rb"(?:\s+|--[^\n]*)*")
    while True:
        p = ws.match(buf, p).end()
        if p >= len(buf):
            return out
        if buf[p] == ord("b") and p + 1 < len(buf) and buf[p + 1] == 2:
            v, p = _binary_value(buf, p)
            out.append(v)
            continue
        # a run of text up to the next binary value (the byte 2 never occurs in text)
        nxt = buf.find(b"b\x02", p)
        text_end = len(buf) if nxt < 0 else nxt
        tp = _TextParser(buf[p:text_end].decode("ascii"))
        while not tp.at_end():
            out.append(tp.value())
        p = text_end


def read_file(path) -> List[Union[np.generic, np.ndarray]]:
    with open(path, "rb") as f:
        return read_values(f.read())


def format_value(v) -> str:
    """Text encoding of one value (scalar or array)."""
    a = np.asarray(v)
    name = _NAME_OF.get(a.dtype)
    if name is None:
        raise TypeError(f"no Futhark type for numpy dtype {a.dtype}")
    if a.ndim and a.size == 0:
        return "empty(" + "".join(f"[{d}]" for d in a.shape) + name + ")"

    def scalar(x) -> str:
        if name == "bool":
            return "true" if x else "false"
        if name.startswith("f"):
            xf = TYPES[name](x)
            if np.isnan(xf):
                return f"{name}.nan"
            if np.isinf(xf):
                return f"{name}.inf" if xf > 0 else f"-{name}.inf"
            r = repr(float(xf)) if name == "f64" else str(xf)
            if "." not in r and "e" not in r and "inf" not in r:
                r += ".0"
            return r + name
        return f"{int(x)}{name}"

    if a.ndim == 0:
        return scalar(a[()])
    flat = [scalar(x) for x in a.reshape(-1).tolist()] if name != "bool" else [scalar(x) for x in a.reshape(-1)]

    def nest(off: int, dims: Sequence[int]) -> str:
        if len(dims) == 1:
            return "[" + ", ".join(flat[off:off + dims[0]]) + "]"
        step = int(np.prod(dims[1:]))
        return "[" + ", ".join(nest(off + i * step, dims[1:]) for i in range(dims[0])) + "]"

    return nest(0, a.shape)


def write_text(values: Iterable, f=None) -> str:
    """Text encoding of several values, one per line; written to f if given."""
    s = "\n".join(format_value(v) for v in values) + "\n"
    if f is not None:
        f.write(s)
    return s


def write_binary(values: Iterable, f: BinaryIO = None) -> bytes:
    """Binary encoding of several values; written to f if given."""
    out = io.BytesIO()
    for v in values:
        a = np.asarray(v)
        name = _NAME_OF.get(a.dtype)
        if name is None:
            raise TypeError(f"no Futhark type for numpy dtype {a.dtype}")
        out.write(b"b\x02" + struct.pack("<b", a.ndim) + name.rjust(4).encode("ascii"))
        if a.ndim:
            out.write(struct.pack(f"<{a.ndim}q", *a.shape))
        out.write(np.ascontiguousarray(a).astype(a.dtype.newbyteorder("<"), copy=False).tobytes())
    b = out.getvalue()
    if f is not None:
        f.write(b)
    return b


def _main(argv=None) -> int:
    import argparse
    ap = argparse.ArgumentParser(description="Convert Futhark value files between text and binary.")
    ap.add_argument("src")
    ap.add_argument("dst")
    ap.add_argument("--to", choices=("text", "binary"), default="binary")
    a = ap.parse_args(argv)
    vals = read_file(a.src)
    if a.to == "text":
        with open(a.dst, "w") as f:
            write_text(vals, f)
    else:
        with open(a.dst, "wb") as f:
            write_binary(vals, f)
    print(" ".join(f"{np.asarray(v).dtype}{list(np.shape(v))}" for v in vals), file=sys.stderr)
    return 0


if __name__ == "__main__":
    sys.exit(_main())
