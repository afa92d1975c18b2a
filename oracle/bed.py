"""TEST INFRASTRUCTURE ONLY: the oracle of the BED ingest.

Restates the reference's BED reading (examples/bed-intersect-si.rs:63-120, parse_bed_line
and read_bed_file): the chrom is the first tab-separated column, start the second, end the
third; the stored end is column 3 - 1 when ``half_open`` (BED ends are exclusive, the index
is end-inclusive); lines with end < 0 or end < start are skipped; intervals are grouped per
chrom.  Where the reference parses without checks (its integer parser folds any byte), this
restatement, like the GPU parser, skips header lines ('#', "track", "browser"), empty lines,
lines with fewer than three columns and non-integer columns, and strips a trailing '\\r'.
Contig ids follow first appearance; line numbers are 0-based over all lines.
"""
from __future__ import annotations


def _int(tok: bytes):
    neg = tok.startswith(b"-")
    digits = tok[1:] if neg else tok
    if not digits or len(digits) > 18 or not digits.isdigit():
        return None
    v = int(digits)
    return -v if neg else v


def _header(line: bytes) -> bool:
    if not line or line.startswith(b"#"):
        return True
    for w in (b"track", b"browser"):
        if line.startswith(w) and (len(line) == len(w) or line[len(w):len(w) + 1] in (b" ", b"\t")):
            return True
    return False


def parse_bed(text: bytes, half_open: bool = True, lo: int = -(2 ** 31), hi: int = 2 ** 31 - 1):
    """Returns (names in first-appearance order, {name: [(start, end, line), ...]}, stats)."""
    lines = text.split(b"\n")
    if text.endswith(b"\n"):
        lines = lines[:-1]
    names, per, st = [], {}, dict(lines=len(lines), intervals=0, skipped_headers=0, malformed=0, filtered=0,
                                   out_of_range=0)
    for k, raw in enumerate(lines):
        line = raw[:-1] if raw.endswith(b"\r") else raw
        if _header(line):
            st["skipped_headers"] += 1
            continue
        f = line.split(b"\t")
        if len(f) < 3 or not f[0]:
            st["malformed"] += 1
            continue
        s, e = _int(f[1]), _int(f[2])
        if s is None or e is None:
            st["malformed"] += 1
            continue
        if half_open:
            e -= 1
        if e < 0 or e < s:
            st["filtered"] += 1
            continue
        if not (lo <= s <= hi and lo <= e <= hi):
            st["out_of_range"] += 1
            continue
        name = f[0].decode("latin-1")
        if name not in per:
            per[name] = []
            names.append(name)
        per[name].append((s, e, k))
        st["intervals"] += 1
    return names, per, st
