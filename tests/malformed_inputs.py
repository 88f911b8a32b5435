"""Reference-sequence and known-SNP files with the irregular rows the
reference's loader (cpp/chromosome.cc:172-221) gives meaning to (test helper).

- FASTA: text before the first header, header descriptions, blank lines,
  CR line ends, a chromosome name repeated with a new sequence (it replaces
  the old one) and one repeated at the end with no sequence (the old one
  stays).
- Known SNPs: rows separated by tabs or spaces, trailing rsIDs, repeated
  positions (the first row counts), unknown chromosomes, blank rows and rows
  of a name alone (the name and position of the row before them stay, and the
  position is decremented again), flags other than 0/1 and frequencies that
  do not parse (the fields after them keep the row before's values), and
  decimals in every plain and non-plain form.

Every position the rows lead to stays inside its chromosome, since the
reference writes its SNP mark without a bounds check."""
import random


def _seq(rng, n):
    return "".join(rng.choice("ACGT") for _ in range(n))


def _lines(s, width=60):
    return [s[i:i + width] for i in range(0, len(s), width)]


def _freqs(rng):
    forms = ["%.4f", "%.4f", "%.17g", "%g", "%.3e"]
    out = []
    for _ in range(4):
        x = rng.choice([0.0, rng.random()])
        out.append(rng.choice(forms) % x)
    return out


def _irregular_freq(rng):
    return rng.choice(["abc", "nan", "inf", "-inf", "1e999", "1e-400", "0x1p-3", ".5", "5.", "+0.25", "-0.0",
                       "0.123456789012345678901234", "1e22", "1e23", "7e-23", "00012.5000", "1e", "--1"])


def snp_rows(rng, lengths, n):
    """n known-SNP rows over chromosomes of the given lengths (1-based
    positions from 10 on, so that a blank row's decrement stays inside)"""
    names = sorted(lengths)
    rows = [""]   # a blank first row: no name yet, nothing is marked
    prev = None   # (name, 1-based pos) of the last row that set both
    for _ in range(n):
        name = rng.choice(names)
        pos = rng.randint(10, lengths[name])
        flags = [str(rng.randint(0, 1)) for _ in range(3)]
        fr = _freqs(rng)
        tail = ["rs%d" % rng.randint(1, 10 ** 6)] if rng.random() < 0.7 else []
        k = rng.random()
        if k < 0.04 and prev:
            rows.append(rng.choice(["", "   ", "\t"]))
            prev = None
            continue
        if k < 0.07 and prev:
            rows.append(prev[0])
            prev = None
            continue
        if k < 0.10:
            rows.append("\t".join(["chrUnknown", str(pos)] + flags + fr))
            prev = None   # its position must not reach a known name
            continue
        if k < 0.15:
            flags[rng.randint(0, 2)] = rng.choice(["2", "x", "01", "-1"])
        elif k < 0.25:
            fr[rng.randint(0, 3)] = _irregular_freq(rng)
        elif k < 0.30 and prev:
            name, pos = prev                    # a repeated position
        elif k < 0.33:
            pos = "+%d" % pos
        sep = " " if rng.random() < 0.2 else "\t"
        rows.append(sep.join([name, str(pos)] + flags + fr + tail))
        prev = (name, int(str(pos).lstrip("+")))
    return rows


def write_loader_inputs(directory, seed):
    """A three-chromosome FASTA and a known-SNP file; returns their paths."""
    rng = random.Random(seed)
    chr1_old, chr1, chr2, chr3 = _seq(rng, 5000), _seq(rng, 4000), _seq(rng, 3000), _seq(rng, 1000)
    chr1 = chr1[:100] + "NNNNnnnnacgt" + chr1[112:]
    fa = ["text before any header", ">chr1 first copy"] + _lines(chr1_old)[:40] + [""] + _lines(chr1_old)[40:]
    fa += [">chr2"] + [x + "\r" for x in _lines(chr2)[:3]] + _lines(chr2)[3:]
    fa += [">chr1\tsecond copy"] + _lines(chr1) + [">chr3"] + _lines(chr3) + [">chr2"]
    lengths = {"chr1": len(chr1), "chr2": len(chr2), "chr3": len(chr3)}
    fasta = directory + "/ref.fa"
    with open(fasta, "w", newline="") as fh:
        fh.write("\n".join(fa) + "\n")
    dbsnp = directory + "/dbsnp.txt"
    with open(dbsnp, "w", newline="") as fh:
        fh.write("\n".join(snp_rows(rng, lengths, 3000)))
    return fasta, dbsnp


def corrupt_workload_inputs(paths, chr_name, genome_len, seed):
    """Append irregular rows to a workload's known-SNP file and, to its FASTA,
    another chromosome and the workload's chromosome repeated with no
    sequence (which leaves its sequence as it was)."""
    rng = random.Random(seed)
    with open(paths["dbsnp"], "a") as fh:
        fh.write("\n".join(snp_rows(rng, {chr_name: genome_len}, 400)) + "\n")
    with open(paths["ref"], "a") as fh:
        fh.write(">chrOther\n" + "\n".join(_lines(_seq(rng, 500))) + "\n>" + chr_name + "\n")
