"""BED ingest: the oracle's parse rules (CPU) and the GPU parser against it."""
import numpy as np
import pytest

from oracle.bed import parse_bed

HAND = (b"track name=x\n#comment\nchr2\t10\t20\tx\nchr1\t5\t6\r\nchr2\t30\t25\nchr1\tx\t9\nchr3\t1\n\n"
        b"chr1\t-5\t0\nchr1\t7\t100\nbrowser position chr1\nchrUn_1\t0\t1\t+\t9\n")


def test_oracle_parse_rules():
    """bed-intersect-si.rs:63-120: chrom / start / end - 1, end < 0 or end < start skipped."""
    names, per, st = parse_bed(HAND)
    assert names == ["chr2", "chr1", "chrUn_1"]
    assert per["chr2"] == [(10, 19, 2)] and per["chr1"] == [(5, 5, 3), (7, 99, 9)]
    assert per["chrUn_1"] == [(0, 0, 11)]
    assert st == dict(lines=12, intervals=4, skipped_headers=4, malformed=2, filtered=2, out_of_range=0)
    names, per, st = parse_bed(HAND, half_open=False)
    assert per["chr2"] == [(10, 20, 2)] and st["filtered"] == 1


def random_bed(seed, n, names, max_pos=2_000_000):
    r = np.random.default_rng(seed)
    lines = [b"# generated", b"track name=t"]
    want = 0
    for k in range(n):
        nm = names[r.integers(len(names))]
        s = int(r.integers(0, max_pos))
        e = s + int(r.integers(1, 5000))
        u = r.random()
        if u < 0.01:
            lines.append(b"")
        elif u < 0.02:
            lines.append(nm.encode() + b"\t%d" % s)                  # two columns: malformed
        elif u < 0.03:
            lines.append(nm.encode() + b"\t%d\t%d" % (e, s))          # end < start: filtered
        elif u < 0.05:
            lines.append(nm.encode() + b"\t%d\t%d\tname\t0\t+\r" % (s, e))
        else:
            lines.append(nm.encode() + b"\t%d\t%d" % (s, e))
            want += 1
    return b"\n".join(lines) + (b"\n" if seed % 2 else b"")


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [32, 64])
def test_gpu_ingest_matches_oracle(bits):
    import __graft_entry__ as g
    g.build()
    from superintervals_gb300 import interval_map as im
    names = ["chr%d" % i for i in (3, 1, 22, 7)] + ["chrX", "chrUn_KI270302v1", "scaffold_" + "9" * 40]
    text = random_bed(7 + bits, 60_000, names)
    onames, per, ost = parse_bed(text)
    idx = im.GpuIndex(bits)
    st = idx.ingest_bed(text)
    assert {k: st[k] for k in ost} == ost
    assert idx.contig_names() == onames
    idx.build()
    s, e, d, _ = idx.arrays()
    seg = np.cumsum([0] + [len(per[n]) for n in onames])
    for c, nm in enumerate(onames):
        rows = sorted(per[nm], key=lambda x: (x[0], -x[1]))         # index order, stable
        got = list(zip(s[seg[c]:seg[c + 1]].tolist(), e[seg[c]:seg[c + 1]].tolist(), d[seg[c]:seg[c + 1]].tolist()))
        assert got == rows
    # queries from BED text on the same contigs (one unknown chrom is skipped)
    qtext = random_bed(99, 5_000, names + ["chrNotThere"])
    _, qper, _ = parse_bed(qtext)
    qs, qe, qc, line, qst = idx.bed_queries(qtext)
    want = sorted((k, onames.index(nm), a, b) for nm, rows in qper.items() if nm in onames for (a, b, k) in rows)
    got = list(zip(line.tolist(), qc.tolist(), qs.tolist(), qe.tolist()))
    assert got == want
    assert qst["unknown_contig"] == len(qper.get("chrNotThere", []))
    # an index image keeps the names
    img = idx.to_bytes()
    other = im.GpuIndex(bits)
    other.from_bytes(img)
    assert other.contig_names() == onames
    idx.close()
    other.close()


@pytest.mark.gpu
def test_gpu_ingest_edge_cases():
    import __graft_entry__ as g
    g.build()
    from superintervals_gb300 import interval_map as im
    idx = im.GpuIndex(32)
    st = idx.ingest_bed(HAND)
    _, _, ost = parse_bed(HAND)
    assert {k: st[k] for k in ost} == ost
    assert idx.contig_names() == ["chr2", "chr1", "chrUn_1"]
    st = idx.ingest_bed(b"chr1\t1\t99999999999\n")              # beyond int32: counted, skipped
    assert st["out_of_range"] == 1 and st["intervals"] == 0
    st = idx.ingest_bed(b"")
    assert st["lines"] == 0
    idx.close()
