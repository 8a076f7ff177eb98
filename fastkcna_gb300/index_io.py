"""Readers of the index files the builds write.

NSG layout (SaveNsg, src/kgraph.cpp:1704-1724): u32 width, u32 entry point,
then per node u32 degree followed by that many u32 ids.

hnswlib layout (written by fasthnsw / fastnsw, src/fasthnsw.cpp:317-342):
a header of size_t offsetLevel0, max_elements, cur_element_count,
size_data_per_element, label_offset, offsetData; int maxlevel; u32 entry
point; size_t maxM, maxM0, M; double mult; size_t ef_construction; then the
level-0 block (per element: u32 link count in its low 16 bits, maxM0 u32 ids,
d floats, size_t label) and per element a u32 byte size followed by its upper
levels' lists (per level: u32 count in the low 16 bits, maxM u32 ids)."""
import struct

import numpy as np

_HNSW_HEADER = struct.Struct("<QQQQQQiIQQQdQ")


def read_nsg(path):
    """(list of uint32 id arrays, entry point, width)."""
    raw = np.fromfile(path, dtype=np.uint32)
    width, ep = int(raw[0]), int(raw[1])
    rows, i = [], 2
    while i < raw.size:
        k = int(raw[i])
        rows.append(raw[i + 1 : i + 1 + k].copy())
        i += 1 + k
    return rows, ep, width


def read_hnswlib(path):
    """Dict with the header fields, `data` (n x d float32, storage order),
    `labels` (n,), `level0` (list of id arrays), `levels` (n,) and `upper`
    (dict level -> list of (node, id array))."""
    buf = open(path, "rb").read()
    h = _HNSW_HEADER.unpack_from(buf, 0)
    keys = ("offset_level0", "max_elements", "cur_element_count", "size_data_per_element", "label_offset",
            "offset_data", "maxlevel", "enterpoint", "maxM", "maxM0", "M", "mult", "ef_construction")
    out = dict(zip(keys, h))
    n, per = out["cur_element_count"], out["size_data_per_element"]
    d = (out["label_offset"] - out["offset_data"]) // 4
    pos = _HNSW_HEADER.size
    blk = np.frombuffer(buf, dtype=np.uint8, count=n * per, offset=pos).reshape(n, per)
    pos += n * per
    cnt0 = blk[:, 0:2].copy().view(np.uint16)[:, 0]
    ids0 = blk[:, 4 : 4 + 4 * out["maxM0"]].copy().view(np.uint32)
    out["level0"] = [ids0[i, : cnt0[i]].copy() for i in range(n)]
    out["data"] = blk[:, out["offset_data"] : out["label_offset"]].copy().view(np.float32).reshape(n, d)
    out["labels"] = blk[:, out["label_offset"] : out["label_offset"] + 8].copy().view(np.uint64)[:, 0]
    per_level = 4 + 4 * out["maxM"]
    levels = np.zeros(n, np.int32)
    upper = {}
    for i in range(n):
        (sz,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        if sz:
            lv = sz // per_level
            levels[i] = lv
            for l in range(1, lv + 1):
                o = pos + (l - 1) * per_level
                (c,) = struct.unpack_from("<H", buf, o)
                ids = np.frombuffer(buf, dtype=np.uint32, count=c, offset=o + 4).copy()
                upper.setdefault(l, []).append((i, ids))
            pos += sz
    out["levels"] = levels
    out["upper"] = upper
    return out
