"""A small CBOR (RFC 8949) encoder/decoder for checkpoints.

The reference writes the whole App with ciborium (src/io.rs:7-18).  serde's
data model maps onto CBOR as follows, and this codec follows it: structs are
maps keyed by field name, tuple structs and tuples are arrays, unit enum
variants are text, other enum variants are single-entry maps {variant:
value}, None is null, f64 is a float (64-bit unless it round-trips through a
shorter form, as ciborium does), integers are the shortest major type 0/1
encoding.  ndarray arrays serialise as {"v": 1, "dim": [..], "data": [..]}.
Tuple map keys (BlockIndex) are arrays.
"""
import math
import struct


class CborError(ValueError):
    pass


class Key(tuple):
    """A hashable array key (serde tuple keys of HashMap)."""


def _head(major: int, n: int) -> bytes:
    if n < 24:
        return bytes([(major << 5) | n])
    if n < 1 << 8:
        return bytes([(major << 5) | 24, n])
    if n < 1 << 16:
        return bytes([(major << 5) | 25]) + struct.pack(">H", n)
    if n < 1 << 32:
        return bytes([(major << 5) | 26]) + struct.pack(">I", n)
    return bytes([(major << 5) | 27]) + struct.pack(">Q", n)


def _float(x: float) -> bytes:
    # the shorter single-precision form when it is exact (half precision is
    # not produced); non-finite values as double
    if math.isfinite(x):
        try:
            f32 = struct.pack(">f", x)
            if struct.unpack(">f", f32)[0] == x:
                return b"\xfa" + f32
        except OverflowError:
            pass
    return b"\xfb" + struct.pack(">d", x)


def dumps(obj) -> bytes:
    out = bytearray()

    def enc(o):
        if o is None:
            out.append(0xF6)
        elif o is True:
            out.append(0xF5)
        elif o is False:
            out.append(0xF4)
        elif isinstance(o, int):
            out.extend(_head(0, o) if o >= 0 else _head(1, -1 - o))
        elif isinstance(o, float):
            out.extend(_float(o))
        elif isinstance(o, str):
            b = o.encode()
            out.extend(_head(3, len(b)))
            out.extend(b)
        elif isinstance(o, (bytes, bytearray)):
            out.extend(_head(2, len(o)))
            out.extend(o)
        elif isinstance(o, (list, tuple)):
            out.extend(_head(4, len(o)))
            for v in o:
                enc(v)
        elif isinstance(o, dict):
            out.extend(_head(5, len(o)))
            for k, v in o.items():
                enc(list(k) if isinstance(k, tuple) else k)
                enc(v)
        else:
            try:
                import numpy as np
                if isinstance(o, np.generic):
                    return enc(o.item())
            except ImportError:
                pass
            raise CborError("cannot encode %r" % type(o))

    enc(obj)
    return bytes(out)


def loads(data: bytes):
    pos = 0

    def need(n):
        nonlocal pos
        if pos + n > len(data):
            raise CborError("truncated")
        b = data[pos:pos + n]
        pos += n
        return b

    def arg(info):
        if info < 24:
            return info
        if info == 24:
            return need(1)[0]
        if info == 25:
            return struct.unpack(">H", need(2))[0]
        if info == 26:
            return struct.unpack(">I", need(4))[0]
        if info == 27:
            return struct.unpack(">Q", need(8))[0]
        raise CborError("indefinite lengths are not supported")

    def dec():
        ib = need(1)[0]
        major, info = ib >> 5, ib & 31
        if major == 0:
            return arg(info)
        if major == 1:
            return -1 - arg(info)
        if major == 2:
            return bytes(need(arg(info)))
        if major == 3:
            return need(arg(info)).decode()
        if major == 4:
            return [dec() for _ in range(arg(info))]
        if major == 5:
            out = {}
            for _ in range(arg(info)):
                k = dec()
                if isinstance(k, list):
                    k = Key(k)
                out[k] = dec()
            return out
        if major == 6:
            arg(info)
            return dec()
        if major == 7:
            if info == 20:
                return False
            if info == 21:
                return True
            if info in (22, 23):
                return None
            if info == 25:
                h = struct.unpack(">e", need(2))[0]
                return float(h)
            if info == 26:
                return struct.unpack(">f", need(4))[0]
            if info == 27:
                return struct.unpack(">d", need(8))[0]
        raise CborError("unsupported item 0x%02x" % ib)

    obj = dec()
    if pos != len(data):
        raise CborError("trailing bytes")
    return obj


def ndarray(shape, data):
    """serde form of an ndarray 0.14 array."""
    return {"v": 1, "dim": list(shape), "data": data}
