"""BAM reader restated from the SAM/BAM specification (§4.1 BGZF, §4.2 records) with Python's zlib:
the CPU check of the device decode (test infrastructure only).  It follows the rules breseq's
htslib-based reading applies (tag accessors src/breseq/alignment.cpp:52-80, read groups
src/breseq/alignment.h:533-607): X1 1 when absent, XL / XR -1 when absent, the first occurrence of
a tag, integer tags of any BAM integer type (other types read as 0), RG as a Z or H string resolved
against the header's @RG IDs (0 when unresolved or with at most one group), and the read file of
(group, mate).  Unplaced records (refID -1) at the end are dropped."""
from __future__ import annotations

import struct
import zlib

import numpy as np


class BamError(ValueError):
    pass


def inflate_bgzf(data: bytes):
    """The concatenated output of every BGZF block, checking each block's CRC-32 and size."""
    out, pos, blocks = [], 0, []
    while pos < len(data):
        if len(data) - pos < 18 or data[pos:pos + 4] != b"\x1f\x8b\x08\x04":
            raise BamError("not a BGZF block")
        xlen = struct.unpack_from("<H", data, pos + 10)[0]
        bsize, x = None, pos + 12
        while x + 4 <= pos + 12 + xlen:
            si1, si2, slen = data[x], data[x + 1], struct.unpack_from("<H", data, x + 2)[0]
            if si1 == 66 and si2 == 67 and slen == 2:
                bsize = struct.unpack_from("<H", data, x + 4)[0]
            x += 4 + slen
        if bsize is None:
            raise BamError("BGZF block without a BC field")
        total = bsize + 1
        cdata = data[pos + 12 + xlen: pos + total - 8]
        crc, isize = struct.unpack_from("<II", data, pos + total - 8)
        raw = zlib.decompress(cdata, -15)
        if len(raw) != isize or (zlib.crc32(raw) & 0xFFFFFFFF) != crc:
            raise BamError("BGZF block size or CRC-32 mismatch")
        blocks.append((sum(len(o) for o in out), isize))
        out.append(raw)
        pos += total
    return b"".join(out), blocks


def read_bam(data: bytes, groups=None):
    """dict(header=..., records=arrays in the bsq_read_soa layout)."""
    stream, _ = inflate_bgzf(data)
    if stream[:4] != b"BAM\1":
        raise BamError("not BAM")
    l_text = struct.unpack_from("<i", stream, 4)[0]
    text = stream[8:8 + l_text].decode()
    o = 8 + l_text
    n_ref = struct.unpack_from("<i", stream, o)[0]
    o += 4
    names, lengths = [], []
    for _ in range(n_ref):
        l_name = struct.unpack_from("<i", stream, o)[0]
        names.append(stream[o + 4:o + 4 + l_name].split(b"\0")[0].decode())
        lengths.append(struct.unpack_from("<i", stream, o + 4 + l_name)[0])
        o += 8 + l_name
    ids, base, count = groups if groups is not None else ([], None, None)
    cols = {k: [] for k in ("tid", "pos", "flag", "mapq", "x1", "xl", "xr", "read_file", "read_group", "l_qseq",
                            "n_cigar", "xj", "isize", "xp", "mtid", "mpos")}
    cig, seq, qual, qnames = [], [], [], []
    seen_unplaced = False
    int_fmt = {"c": "<b", "C": "<B", "s": "<h", "S": "<H", "i": "<i", "I": "<I"}
    fixed = {"A": 1, "c": 1, "C": 1, "s": 2, "S": 2, "i": 4, "I": 4, "f": 4}
    while o < len(stream):
        bs = struct.unpack_from("<i", stream, o)[0]
        o_rec = o
        end = o + 4 + bs
        ref_id, pos, l_name, mapq, _bin, n_cig, flag, l_seq = struct.unpack_from("<iiBBHHHi", stream, o + 4)
        c0 = o + 36 + l_name
        s0 = c0 + 4 * n_cig
        q0 = s0 + (l_seq + 1) // 2
        a = q0 + l_seq
        tags = {}
        while a < end:
            tag, typ = stream[a:a + 2].decode(), chr(stream[a + 2])
            a += 3
            if typ in fixed:
                size = fixed[typ]
            elif typ in "ZH":
                size = stream.index(b"\0", a) - a + 1
            elif typ == "B":
                sub, cnt = chr(stream[a]), struct.unpack_from("<I", stream, a + 1)[0]
                size = 5 + cnt * {"c": 1, "C": 1, "s": 2, "S": 2, "i": 4, "I": 4, "f": 4}[sub]
            else:
                raise BamError("unknown aux type")
            if tag not in tags:
                tags[tag] = (typ, stream[a:a + size])
            a += size
        o = end
        # a CIGAR of more than 65535 operations kept in CG:B:I behind the placeholder <l_seq>S<len>N
        # (SAM specification 4.2.2): the library's records hold 65535 operations at most, so it is refused
        if "CG" in tags and tags["CG"][0] == "B" and tags["CG"][1][:1] == b"I" and n_cig == 2:
            c1, c2 = struct.unpack_from("<II", stream, c0)
            if c1 == (l_seq << 4) | 4 and (c2 & 0xF) == 3:
                raise BamError("a CIGAR of more than 65535 operations kept in the CG tag")
        if ref_id < 0:
            seen_unplaced = True
            continue
        if seen_unplaced:
            raise BamError("unplaced records before placed ones")

        def as_int(t, default):
            if t not in tags:
                return default
            typ, v = tags[t]
            return struct.unpack(int_fmt[typ], v[:struct.calcsize(int_fmt[typ])])[0] if typ in int_fmt else 0

        group = 0
        if "RG" in tags and len(ids) > 1 and tags["RG"][0] in "ZH":
            rg = tags["RG"][1][:-1].decode()
            group = ids.index(rg) if rg in ids else 0
        rfile = 0
        if ids and base is not None and group < len(ids) and count[group] > 0:
            rfile = base[group] + (1 if (flag & 0x80) and count[group] > 1 else 0)
        # XP: the pair orientation breseq writes as a Z string (resolve_alignments.cpp:1255-1273); anything
        # else, or no tag, is no orientation (3)
        xp = 3
        if "XP" in tags and tags["XP"][0] in "ZH":
            xp = {b"FR\0": 0, b"RF\0": 1, b"FF\0": 2}.get(bytes(tags["XP"][1]), 3)
        mtid, mpos, tlen = struct.unpack_from("<iii", stream, o_rec + 24)
        for k, v in (("tid", ref_id), ("pos", pos), ("flag", flag), ("mapq", mapq),
                     ("x1", as_int("X1", 1) & 0xFFFFFFFF), ("xl", as_int("XL", -1)), ("xr", as_int("XR", -1)),
                     ("read_file", rfile), ("read_group", group), ("l_qseq", l_seq), ("n_cigar", n_cig),
                     ("xj", 1 if "XJ" in tags else 0), ("isize", tlen), ("xp", xp), ("mtid", mtid), ("mpos", mpos)):
            cols[k].append(v)
        qnames.append(stream[o_rec + 36:o_rec + 36 + l_name - 1])
        cig.append(np.frombuffer(stream[c0:s0], dtype="<u4"))
        sq = stream[s0:q0]
        ql = stream[q0:q0 + l_seq] + (b"\0" if l_seq & 1 else b"")
        seq.append(np.frombuffer(sq, dtype=np.uint8))
        qual.append(np.frombuffer(ql, dtype=np.uint8))
    dts = dict(tid=np.int32, pos=np.int32, flag=np.uint16, mapq=np.uint8, x1=np.uint32, xl=np.int32, xr=np.int32,
               read_file=np.uint8, read_group=np.uint16, l_qseq=np.uint32, n_cigar=np.uint16, xj=np.uint8,
               isize=np.int32, xp=np.uint8, mtid=np.int32, mpos=np.int32)
    rec = {k: np.array(v, dtype=dts[k]) for k, v in cols.items()}
    nc = rec["n_cigar"].astype(np.uint64)
    rec["cigar_off"] = np.concatenate([[0], np.cumsum(nc)[:-1]]).astype(np.uint64) if len(nc) else np.zeros(0, np.uint64)
    nib = rec["l_qseq"].astype(np.uint64) + (rec["l_qseq"].astype(np.uint64) & 1)
    rec["seq_off"] = np.concatenate([[0], np.cumsum(nib)[:-1]]).astype(np.uint64) if len(nib) else np.zeros(0, np.uint64)
    rec["cigar"] = np.concatenate(cig).astype(np.uint32) if cig else np.zeros(0, np.uint32)
    rec["seq"] = np.concatenate(seq) if seq else np.zeros(0, np.uint8)
    rec["qual"] = np.concatenate(qual) if qual else np.zeros(0, np.uint8)
    rec["qname_off"] = np.concatenate([[0], np.cumsum([len(x) for x in qnames])]).astype(np.uint64)
    rec["qname"] = np.frombuffer(b"".join(qnames), dtype=np.uint8).copy()
    return dict(header=dict(text=text, names=names, lengths=lengths), records=rec)
