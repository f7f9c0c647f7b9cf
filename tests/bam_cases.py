"""Hand-made BAM files for the decode tests: tags of every integer type and of other types, repeated
tags, unknown read groups, a single read group, unplaced records."""
import struct

import numpy as np

from breseq_gb300 import synth


def record(ref_id, pos, cigar_ops, seq, tags=b"", flag=0, mapq=42, name=b"r"):
    ops = {"M": 0, "I": 1, "D": 2, "N": 3, "S": 4, "H": 5, "P": 6, "=": 7, "X": 8}
    cig = b"".join(struct.pack("<I", (n << 4) | ops[o]) for n, o in cigar_ops)
    nib = {"A": 1, "C": 2, "G": 4, "T": 8, "N": 15}
    codes = [nib[c] for c in seq] + ([0] if len(seq) & 1 else [])
    packed = bytes((codes[i] << 4) | codes[i + 1] for i in range(0, len(codes), 2))
    qual = bytes([30] * len(seq))
    body = struct.pack("<iiBBHHHiiii", ref_id, pos, len(name) + 1, mapq, 4680, len(cigar_ops), flag, len(seq), -1, -1, 0)
    rec = body + name + b"\0" + cig + packed + qual + tags
    return struct.pack("<i", len(rec)) + rec


def bam(records, targets=(("chrA", 1000), ("chrB", 500)), rg_ids=("g0", "g1"), block_payload=0xFF00, split=False):
    text = "@HD\tVN:1.6\tSO:coordinate\n" + "".join(f"@SQ\tSN:{n}\tLN:{l}\n" for n, l in targets)
    text += "".join(f"@RG\tID:{g}\tLB:{g}\n" for g in rg_ids)
    head = b"BAM\1" + struct.pack("<i", len(text)) + text.encode() + struct.pack("<i", len(targets))
    for n, l in targets:
        head += struct.pack("<i", len(n) + 1) + n.encode() + b"\0" + struct.pack("<i", l)
    out = [synth._bgzf_block(head, 6)]
    body = b"".join(records)
    if split:   # cut the record stream at an arbitrary point: records span blocks
        cut = len(body) // 2 + 7
        out += [synth._bgzf_block(body[:cut], 6), synth._bgzf_block(body[cut:], 6)]
    else:
        buf = b""
        for r in records:
            if len(buf) + len(r) > block_payload and buf:
                out.append(synth._bgzf_block(buf, 6))
                buf = b""
            buf += r
        if buf:
            out.append(synth._bgzf_block(buf, 6))
    out.append(synth.BGZF_EOF)
    return b"".join(out)


def tag_cases():
    """Records exercising the tag rules; returns (bam bytes, groups)."""
    i = lambda t, c, fmt, v: t + c + struct.pack(fmt, v)
    recs = [
        record(0, 10, [(20, "M")], "ACGT" * 5, i(b"X1", b"C", "<B", 3) + b"RGZg1\0"),
        record(0, 12, [(20, "M")], "ACGT" * 5, i(b"X1", b"S", "<H", 2) + i(b"X1", b"C", "<B", 9) + b"RGZg0\0", flag=0x80 | 0x1),
        record(0, 14, [(2, "S"), (18, "M")], "ACGT" * 5, i(b"XL", b"c", "<b", 2) + i(b"XR", b"s", "<h", 4) + b"RGZzz\0"),
        record(0, 16, [(20, "M")], "ACGTA" * 4, b"X1f" + struct.pack("<f", 2.0) + b"XJi" + struct.pack("<i", 1)),
        record(0, 18, [(10, "M"), (2, "I"), (9, "M")], "ACGTACGTACGTACGTACGTA", b"NMi" + struct.pack("<i", 2) +
               b"ZBBi" + struct.pack("<I", 2) + struct.pack("<2i", 7, 8) + i(b"XR", b"I", "<I", 6) + b"RGAq"),
        record(1, 5, [(21, "M")], "ACGTACGTACGTACGTACGTA", b"RGHg1\0" + i(b"X1", b"i", "<i", 4), flag=0x80 | 0x1),
        record(-1, -1, [], "ACGT", flag=0x4),
        record(-1, -1, [], "ACG", flag=0x4),
    ]
    return recs, (["g0", "g1"], [0, 2], [2, 1])
