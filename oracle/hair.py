"""TEST INFRASTRUCTURE ONLY: the CPU oracle of the `.hair` file format and of
strand reduction, restated from the reference (pinned against the
reference's own code in oracle/_ref by tests/test_oracle_hair.py).

- read_hair / write_hair: HairStyle::load / save (src/vkhr/scene_graph/
  hair_style.cc:24-70, field readers :576-623, writers :625-665; the 128-byte
  FileHeader of include/vkhr/scene_graph/hair_style.hh:147-174).
- reduce_select / reduce: HairStyle::reduce (hair_style.cc:375-449) with its
  xorshift64 (:679-685), HairStyle::shuffle = reduce(1) (:371-373).
"""
import struct

import numpy as np

FIELDS = ("segments", "vertices", "thickness", "transparency", "color", "tangents", "indices", "bounding_box")
_HEADER = struct.Struct("<4sIII I ff 3f 64s 3f 3f")  # 128 bytes
assert _HEADER.size == 128


def read_header(path):
    with open(path, "rb") as f:
        raw = f.read(128)
    if len(raw) != 128:
        raise ValueError("reading the file header")
    (sig, strands, verts, bits, default_segments, thick, transp, c0, c1, c2, info, b0, b1, b2, b3, b4, b5) = \
        _HEADER.unpack(raw)
    return {"signature": sig, "strand_count": strands, "vertex_count": verts, "fields": bits,
            "default_segment_count": default_segments, "default_thickness": thick, "default_transparency": transp,
            "default_color": (c0, c1, c2), "information": info, "bounding_box_min": (b0, b1, b2),
            "bounding_box_max": (b3, b4, b5)}


def read_hair(path):
    """HairStyle::load: the header and every array the header's fields announce,
    in the file's order (segments u16 per strand; vertices, color, tangents
    float3 per vertex; thickness, transparency float per vertex; indices u32,
    2 per segment = 2 * (vertices - strands))."""
    h = read_header(path)
    if h["signature"] != b"HAIR":
        raise ValueError("invalid signature")
    n, v, bits = h["strand_count"], h["vertex_count"], h["fields"]
    out = {"header": h}
    with open(path, "rb") as f:
        f.seek(128)
        if bits & 1:
            out["segments"] = np.frombuffer(f.read(2 * n), dtype="<u2").copy()
        if bits & 2:
            out["vertices"] = np.frombuffer(f.read(12 * v), dtype="<f4").reshape(-1, 3).copy()
        if bits & 4:
            out["thickness"] = np.frombuffer(f.read(4 * v), dtype="<f4").copy()
        if bits & 8:
            out["transparency"] = np.frombuffer(f.read(4 * v), dtype="<f4").copy()
        if bits & 16:
            out["color"] = np.frombuffer(f.read(12 * v), dtype="<f4").reshape(-1, 3).copy()
        if bits & 32:
            out["tangents"] = np.frombuffer(f.read(12 * v), dtype="<f4").reshape(-1, 3).copy()
        if bits & 64:
            strands = len(out["segments"]) if "segments" in out else n
            out["indices"] = np.frombuffer(f.read(4 * 2 * (v - strands)), dtype="<u4").copy()
    for k, size in (("segments", 2 * n), ("vertices", 12 * v)):
        if k in out and out[k].nbytes != size:
            raise ValueError("reading " + k)
    if "vertices" not in out:
        raise ValueError("invalid format: no vertices")
    return out


def write_hair(path, vertices, segments=None, tangents=None, indices=None, thickness=None, transparency=None,
               color=None, default_segment_count=0, information=b""):
    """A `.hair` file in HairStyle::save's layout (header completed as
    complete_header does: signature, field bits, counts)."""
    v = np.ascontiguousarray(vertices, dtype="<f4").reshape(-1, 3)
    n = len(segments) if segments is not None else 0
    arrays = [segments, v, thickness, transparency, color, tangents, indices]
    bits = 0
    for i, a in enumerate(arrays):
        if a is not None and len(a):
            bits |= 1 << i
    hdr = _HEADER.pack(b"HAIR", n, len(v), bits, default_segment_count, 0.0, 0.0, 0.0, 0.0, 0.0,
                       information.ljust(64, b"\0")[:64], 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
    dtypes = ["<u2", "<f4", "<f4", "<f4", "<f4", "<f4", "<u4"]
    with open(path, "wb") as f:
        f.write(hdr)
        for a, dt in zip(arrays, dtypes):
            if a is not None and len(a):
                f.write(np.ascontiguousarray(a, dtype=dt).tobytes())


_M64 = (1 << 64) - 1


def xorshift64(state):
    """hair_style.cc:679-685: x ^= x << 13; x ^= x >> 7; x ^= x << 17 (64-bit)."""
    x = state
    x ^= (x << 13) & _M64
    x ^= x >> 7
    x ^= (x << 17) & _M64
    return x


def reduce_select(strand_count, ratio, seed, segments=None, default_segment_count=0):
    """HairStyle::reduce's strand choice: (the original strand of every kept
    strand, in the order kept; the seed after; the kept strands' segment
    counts).  Its arithmetic as the reference does it: strands_left =
    strand_count - ceil(strand_count * ratio) with the product in FP32, the
    `while (--strands_left && ...)` pre-decrement of an unsigned (so 0 wraps
    and every strand is kept, shuffled: ratio 1 is HairStyle::shuffle), each
    pick xorshift64(seed) / double(2^64 - 1) * remaining, truncated, then a
    swap-with-last removal of the strand from both lists."""
    prod = np.float32(np.float32(strand_count) * np.float32(ratio))
    left_f = np.float32(np.float32(strand_count) - np.float32(np.ceil(prod)))
    strands_left = int(left_f) & 0xFFFFFFFF  # unsigned conversion of the FP32 difference
    # Python ints: numpy's uint16 would wrap the running vertex offset at 65,536
    segs = [int(x) for x in segments] if segments is not None and len(segments) else None
    offsets = []
    acc = 0
    for i in range(strand_count):
        offsets.append(acc)
        acc += (segs[i] if segs is not None else default_segment_count) + 1
    ids = list(range(strand_count))
    order, kept = [], []
    state = seed & _M64
    while True:
        strands_left = (strands_left - 1) & 0xFFFFFFFF
        if not (strands_left and len(offsets)):
            break
        state = xorshift64(state)
        r = float(state) / float(_M64)
        k = int(r * len(offsets))
        sc = default_segment_count
        if segs is not None:
            sc = segs[k]
            segs[k], segs[-1] = segs[-1], segs[k]
            segs.pop()
        kept.append(sc)
        order.append((ids[k], offsets[k], sc))
        offsets[k], offsets[-1] = offsets[-1], offsets[k]
        ids[k], ids[-1] = ids[-1], ids[k]
        offsets.pop()
        ids.pop()
    return order, state, kept


def reduce(vertices, tangents, strand_count, ratio, seed, segments=None, default_segment_count=0):
    """HairStyle::reduce on arrays: the kept strands' vertices and tangents in
    the order kept, their segment counts, and the seed after."""
    order, state, kept = reduce_select(strand_count, ratio, seed, segments, default_segment_count)
    rows = [np.arange(start, start + sc + 1) for _, start, sc in order]
    idx = np.concatenate(rows) if rows else np.zeros(0, dtype=np.int64)
    v = np.asarray(vertices)[idx]
    t = np.asarray(tangents)[idx] if tangents is not None else None
    return v, t, np.asarray(kept, dtype=np.uint16), state
