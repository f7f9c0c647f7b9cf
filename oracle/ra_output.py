"""CPU restatement of the output side of breseq's scoring path (test infrastructure only).

  - formatting of RA fields                 src/breseq/identify_mutations.cpp:1836-1910, common.h:845-870
  - test_RA_evidence and its filters        src/breseq/identify_mutations.cpp:143-749
  - error_rates.tab                         src/breseq/error_count.cpp:660-690, 1005-1026
  - base_qual_error_prob.#.tab              src/breseq/error_count.cpp:697-785
  - unique_only_coverage_distribution.tab   src/breseq/error_count.cpp:239-253
  - GenomeDiff RA / MC / UN lines, ids in add order, cGenomeDiff sort
                                            src/breseq/genome_diff.cpp:685-760, genome_diff_entry.cpp:570-660

Pure Python over a few hundred items; it checks the library's C++ output code byte for byte.
"""
from __future__ import annotations

import math

CH = "ACGT.N"

CONSENSUS_DEFAULTS = dict(polymorphism_prediction=0, polymorphism_precision_places=3, mutation_log10_e_value_cutoff=10.0,
                          consensus_frequency_cutoff=0.5, polymorphism_log10_e_value_cutoff=10.0,
                          polymorphism_frequency_cutoff=0.10, polymorphism_minimum_variant_coverage_each_strand=2.0,
                          polymorphism_fisher_strand_p_value_cutoff=0.05)
POLYMORPHISM_DEFAULTS = dict(polymorphism_prediction=1, polymorphism_precision_places=8, mutation_log10_e_value_cutoff=10.0,
                             consensus_frequency_cutoff=0.95, polymorphism_log10_e_value_cutoff=2.0,
                             polymorphism_frequency_cutoff=0.05, polymorphism_minimum_variant_coverage_each_strand=2.0,
                             polymorphism_fisher_strand_p_value_cutoff=0.05)
ALL_KEYS = ["consensus_minimum_variant_coverage", "consensus_minimum_total_coverage",
            "consensus_minimum_variant_coverage_each_strand", "consensus_minimum_total_coverage_each_strand",
            "consensus_reject_indel_homopolymer_length", "consensus_reject_surrounding_homopolymer_length",
            "polymorphism_minimum_variant_coverage", "polymorphism_minimum_total_coverage",
            "polymorphism_minimum_total_coverage_each_strand", "polymorphism_reject_indel_homopolymer_length",
            "polymorphism_reject_surrounding_homopolymer_length", "polymorphism_ks_quality_p_value_cutoff",
            "polymorphism_no_indels"]


def settings(polymorphism: bool, **over):
    s = dict(POLYMORPHISM_DEFAULTS if polymorphism else CONSENSUS_DEFAULTS)
    for k in ALL_KEYS:
        s.setdefault(k, 0)
    s.update(over)
    return s


def fmt(v, precision, scientific):
    if v is None or (isinstance(v, float) and math.isnan(v)):
        return "NA"
    s = ("%.*e" if scientific else "%.*f") % (precision, v)
    if scientific and len(s) >= 3 and s[-3] == "0":
        s = s[:-3] + s[-2:]
    return s


def fmt_default(v):
    return "%g" % v


def _num(s):
    try:
        return float(s)
    except ValueError:
        return 0.0


def ra_fields(r, seq_id, places):
    def reported(f):
        return 0.0 if (r["n"] == 0 or f < 0.5 / r["n"]) else f
    spec = ",".join(f"{CH[b]}:{fmt(reported(r['f'][b]), places, True)}" for b in range(5) if reported(r["f"][b]) > 0.0)
    e = {"seq_id": seq_id, "position": str(r["position"]), "insert_position": str(r["insert_position"]),
         "score": fmt(r["score"], 1, False), "ref_base": r["ref_base"], "new_base": r["new_base"],
         "major_base": r["major_base"], "minor_base": r["minor_base"],
         "major_frequency": fmt(r["major_frequency"], places, True), "frequency": fmt(r["frequency"], places, True),
         "allele_frequencies": spec, "frequency_lower": fmt(r["frequency_lower"], places, True),
         "frequency_upper": fmt(r["frequency_upper"], places, True),
         "ks_quality_p_value": fmt(r["ks_quality_p"], 5, True), "fisher_strand_p_value": fmt(r["fisher_strand_p"], 5, True)}
    for k in ("ref_cov", "new_cov", "major_cov", "minor_cov", "total_cov"):
        e[k] = f"{r[k][0]}/{r[k][1]}"
    return e


def _reject(e, reason, field="reject"):
    if field not in e:
        e[field] = reason
    elif reason not in e[field].split(","):
        e[field] += "," + reason


def _cov(e, k):
    a, b = e[k].split("/")
    return _num(a), _num(b)


def _homopolymer(e, seq, indel_len, surround_len, no_indels):
    L = len(seq)

    def base(p):
        return seq[p - 1] if 1 <= p <= L else ""
    if indel_len and (e["ref_base"] == "." or e["new_base"] == "."):
        mut_pos = int(e["position"])
        is_ins = _num(e["insert_position"]) > 0
        mut_base = e["new_base"] if e["ref_base"] == "." else e["ref_base"]
        hl = 0
        no_match = False
        if is_ins and base(mut_pos) != mut_base:
            mut_pos += 1
            if mut_pos > L or base(mut_pos) != mut_base:
                no_match = True
        if not no_match:
            sp = mut_pos - 1
            while base(sp) == mut_base and sp > 0:
                sp -= 1
            sp += 1
            ep = mut_pos + 1
            while base(ep) == mut_base and ep <= L:
                ep += 1
            ep -= 1
            hl = ep - sp + 1
        if hl >= indel_len:
            _reject(e, "INDEL_HOMOPOLYMER")
    if surround_len and e["ref_base"] != "." and e["new_base"] != ".":
        mut_pos = int(e["position"])
        mb = e["new_base"]
        sp = mut_pos - 1
        while sp >= 1 and base(sp) == mb:
            sp -= 1
        sp += 1
        ep = mut_pos + 1
        while ep <= L and base(ep) == mb:
            ep += 1
        ep -= 1
        if sp < mut_pos and ep > mut_pos and ep - sp + 1 >= surround_len:
            _reject(e, "SURROUNDING_HOMOPOLYMER")
    if no_indels and (e["ref_base"] == "." or e["new_base"] == "."):
        _reject(e, "POLYMORPHIC_INDEL")


def classify(e, seq, s):
    """test_RA_evidence_CONSENSUS_mode / _POLYMORPHISM_mode; returns True when the entry is deleted."""
    sc = e.get("score", "NA")
    score = float("nan") if sc.upper() in ("NA", "#NA", "NAN") else _num(sc)
    lower, upper = _num(e["frequency_lower"]), _num(e["frequency_upper"])
    poly = bool(s["polymorphism_prediction"])
    if score < s["mutation_log10_e_value_cutoff"]:
        _reject(e, "SCORE_CUTOFF")
    bound = upper if poly else lower
    if s["consensus_frequency_cutoff"] > 0.0 and bound < s["consensus_frequency_cutoff"]:
        _reject(e, "FREQUENCY_CUTOFF")
    if s["consensus_minimum_variant_coverage_each_strand"] > 0:
        t, b = _cov(e, "major_cov")
        if t < s["consensus_minimum_variant_coverage_each_strand"] or b < s["consensus_minimum_variant_coverage_each_strand"]:
            _reject(e, "VARIANT_STRAND_COVERAGE")
    if s["consensus_minimum_total_coverage_each_strand"] > 0:
        t, b = _cov(e, "total_cov")
        if t < s["consensus_minimum_total_coverage_each_strand"] or b < s["consensus_minimum_total_coverage_each_strand"]:
            _reject(e, "TOTAL_STRAND_COVERAGE")
    if s["consensus_minimum_variant_coverage"] > 0 and sum(_cov(e, "major_cov")) < s["consensus_minimum_variant_coverage"]:
        _reject(e, "VARIANT_COVERAGE")
    if s["consensus_minimum_total_coverage"] > 0 and sum(_cov(e, "total_cov")) < s["consensus_minimum_total_coverage"]:
        _reject(e, "TOTAL_COVERAGE")
    _homopolymer(e, seq, s["consensus_reject_indel_homopolymer_length"],
                 s["consensus_reject_surrounding_homopolymer_length"], False)
    if "reject" not in e:
        e["prediction"] = "consensus"
        return e["ref_base"] == e["major_base"]
    e["consensus_reject"] = e.pop("reject")
    if score < s["polymorphism_log10_e_value_cutoff"]:
        _reject(e, "SCORE_CUTOFF")
    if s["polymorphism_frequency_cutoff"] > 0.0 and lower < s["polymorphism_frequency_cutoff"]:
        _reject(e, "FREQUENCY_CUTOFF")
    if s["polymorphism_ks_quality_p_value_cutoff"] and _num(e["ks_quality_p_value"]) < s["polymorphism_ks_quality_p_value_cutoff"]:
        _reject(e, "KS_BASE_QUALITY")
    if s["polymorphism_fisher_strand_p_value_cutoff"] and _num(e["fisher_strand_p_value"]) < s["polymorphism_fisher_strand_p_value_cutoff"]:
        _reject(e, "FISHER_STRAND")
    m = s["polymorphism_minimum_variant_coverage_each_strand"]
    if m > 0:
        maj_var = e["major_base"] != e["ref_base"]
        min_var = e["minor_base"] != e["ref_base"]
        if not maj_var and not min_var:
            maj_var = min_var = True
        ok = True
        if maj_var:
            t, b = _cov(e, "major_cov")
            ok = ok and t >= m and b >= m
        if min_var:
            t, b = _cov(e, "minor_cov")
            ok = ok and t >= m and b >= m
        if not ok:
            _reject(e, "VARIANT_STRAND_COVERAGE")
    m = s["polymorphism_minimum_total_coverage_each_strand"]
    if m > 0:
        t, b = _cov(e, "total_cov")
        if not (t >= m and b >= m):
            _reject(e, "TOTAL_STRAND_COVERAGE")
    m = s["polymorphism_minimum_variant_coverage"]
    if m > 0 and not (sum(_cov(e, "major_cov")) >= m and sum(_cov(e, "minor_cov")) >= m):
        _reject(e, "VARIANT_COVERAGE")
    m = s["polymorphism_minimum_total_coverage"]
    if m > 0 and sum(_cov(e, "total_cov")) < m:
        _reject(e, "TOTAL_COVERAGE")
    _homopolymer(e, seq, s["polymorphism_reject_indel_homopolymer_length"],
                 s["polymorphism_reject_surrounding_homopolymer_length"], bool(s["polymorphism_no_indels"]))
    if "reject" not in e:
        e["prediction"] = "polymorphism"
        return False
    if not poly:
        e["polymorphism_reject"] = e.pop("reject")
        return True
    e["prediction"] = "polymorphism"
    return False


def classify_all(ra, sample, s):
    out = []
    for r in ra:
        t = r["tid"]
        seq = bytes(sample.ref_seq[int(sample.target_offset[t]):int(sample.target_offset[t + 1])]).decode()
        e = ra_fields(r, sample.target_names[t], s["polymorphism_precision_places"])
        deleted = classify(e, seq, s)
        out.append(dict(deleted=deleted, prediction=e.get("prediction", ""), reject=e.get("reject", ""),
                        consensus_reject=e.get("consensus_reject", ""),
                        polymorphism_reject=e.get("polymorphism_reject", "")))
    return out


def error_rates_text(counts, R, Q, log10_table):
    lines = [f"read_set={R},ref_base,obs_base,quality={Q}", "read_set\tref_base\tobs_base\tquality\tlog10_probability"]
    for idx in range(R * 25 * Q):
        rs, ref, obs, q = idx % R, (idx // R) % 5, (idx // (5 * R)) % 5, idx // (25 * R)
        lines.append(f"{rs}\t{CH[ref]}\t{CH[obs]}\t{q}\t{fmt_default(log10_table[idx])}")
    return "\n".join(lines) + "\n"


def coverage_distribution_text(hist, size):
    return "coverage\tn\n" + "".join(f"{j}\t{int(hist[j])}\n" for j in range(1, size))


def base_qual_texts(counts, R, Q):
    t = [0.0] * (R * Q * 25)
    for idx in range(R * 25 * Q):
        rs, ref, obs, q = idx % R, (idx // R) % 5, (idx // (5 * R)) % 5, idx // (25 * R)
        t[rs * 25 * Q + q * 25 + obs * 5 + ref] += float(counts[idx])
    texts = []
    running = 0.0
    for r in range(R):
        for k in range(25 * Q):
            i = r * 25 * Q + k
            running += t[i]
            if i % 5 == 4:
                for j in range(i - 4, i + 1):
                    if running > 0:
                        t[j] /= running
                    if t[j] == 0:
                        t[j] = float("nan")
                running = 0.0
        rows = ["quality" + "".join(f"\t{CH[b1]}{CH[b2]}" for b1 in range(5) for b2 in range(5))]
        for q in range(Q):
            vals = []
            for b1 in range(5):
                for b2 in range(5):
                    v = t[r * 25 * Q + q * 25 + b1 * 5 + b2]
                    vals.append("NA" if math.isnan(v) else fmt_default(v))
            rows.append(str(q) + "".join("\t" + v for v in vals))
        texts.append("\n".join(rows) + "\n")
    return texts


def gd_text(sample, prop_cutoff, places, ra, calls, mc, un):
    names = sample.target_names
    order = list(sample.target_order)
    rank = {t: i for i, t in enumerate(order)}
    lens = [int(sample.target_offset[t + 1] - sample.target_offset[t]) for t in range(len(names))]
    items = []
    for i, r in enumerate(ra):
        if calls is not None and calls[i]["deleted"]:
            continue
        e = ra_fields(r, names[r["tid"]], places)
        if calls is not None:
            for k in ("prediction", "reject", "consensus_reject", "polymorphism_reject"):
                if calls[i][k]:
                    e[k] = calls[i][k]
        items.append(dict(type=0, tid=r["tid"], add=(rank[r["tid"]], r["position"], 2, r["insert_position"]), e=e))
    for m in mc:
        whole = prop_cutoff[m["tid"]] < 0
        e = {"seq_id": names[m["tid"]], "start": str(m["start"]), "end": str(m["end"]), "start_range": str(m["start_range"]),
             "end_range": str(m["end_range"])}
        for k in ("left_outside_cov", "left_inside_cov", "right_inside_cov", "right_outside_cov"):
            e[k] = fmt(m[k], 0, False)
        add = (rank[m["tid"]], lens[m["tid"]] + 1, 3, 0) if whole else (rank[m["tid"]], m["end"] + 1, 0, 0)
        items.append(dict(type=1, tid=m["tid"], add=add, e=e))
    for u in un:
        e = {"seq_id": names[u["tid"]], "start": str(u["start"]), "end": str(u["end"])}
        items.append(dict(type=2, tid=u["tid"], add=(rank[u["tid"]], u["end"] + 1, 1, 0), e=e))
    for i, it in enumerate(sorted(items, key=lambda x: x["add"])):
        it["id"] = i + 1
    group = {0: 3, 1: 4, 2: 7}

    def key(it):
        e = it["e"]
        pos = int(e["position"] if it["type"] == 0 else e["start"])
        if it["type"] == 0:
            rest = (e["insert_position"], e["ref_base"], e["new_base"])
        elif it["type"] == 1:
            rest = (int(e["end"]), e["start_range"], e["end_range"])
        else:
            rest = (int(e["end"]),)
        return (group[it["type"]], e["seq_id"], pos, rest)
    insertion = sorted(items, key=lambda x: x["add"])
    out = ["#=GENOME_DIFF\t1.0"]
    spec = {0: ["seq_id", "position", "insert_position", "ref_base", "new_base"],
            1: ["seq_id", "start", "end", "start_range", "end_range"], 2: ["seq_id", "start", "end"]}
    for it in sorted(insertion, key=key):
        e = dict(it["e"])
        cols = [("RA", "MC", "UN")[it["type"]], str(it["id"]), "."] + [e.pop(f) for f in spec[it["type"]]]
        cols += [f"{k}={v}" for k, v in sorted(e.items()) if v and not k.startswith("_")]
        out.append("\t".join(cols))
    return "\n".join(out) + "\n"
