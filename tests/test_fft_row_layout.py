"""Shared-memory layout of the FP32 row transforms (axg_fft_ff.cu: fswz,
rowline_pitch, f_stockham's passes).

Model: a half warp's 8-byte requests are served in one wavefront per
distinct 4-byte word of the most-used bank.  For every access pattern of the
radix-8 Stockham line transform (first-pass reads, the exchanges' writes and
reads, the last pass's stores) the swizzled, pitched layout must need the
minimum, 2 wavefronts per warp instruction, at every line length the
library uses (M = 8 .. 256 points), and the swizzle must permute each line.
The i + i / 8 padding it replaced needed 160 wavefronts per line where 96
suffice (M >= 128)."""


def fswz(i):
    return i ^ ((i >> 3) & 15)


def pitch(m):
    return m if m >= 128 else m + m // 8


def wavefronts(word_addrs):
    per_bank = {}
    for a in word_addrs:
        per_bank.setdefault(a % 32, set()).add(a)
    return max(len(s) for s in per_bank.values())


def patterns(L):
    """Per warp instruction, the element index each lane touches; TH = L / 8
    lanes per line, so a warp covers 32 / TH lines (or part of one)."""
    TH = max(L // 8, 1)
    lanes = [(lane // TH, lane % TH) for lane in range(32)]
    out, NS = [], 1
    while True:
        R = 8 if L // NS >= 8 else L // NS
        NI = 8 // R
        for q in range(NI):
            for r in range(R):
                out.append([(ln, j + q * TH + r * (L // R)) for ln, j in lanes])
        if NS * R == L:
            for q in range(NI):
                for r in range(R):
                    out.append([(ln, j + q * TH + r * NS) for ln, j in lanes])
            return out
        for q in range(NI):
            for r in range(R):
                w = []
                for ln, j in lanes:
                    jj = j + q * TH
                    w.append((ln, (jj // NS) * NS * R + (jj % NS) + r * NS))
                out.append(w)
        NS *= R


def cost(L, index, lp):
    total = 0
    for inst in patterns(L):
        for half in (inst[:16], inst[16:]):
            words = []
            for ln, e in half:
                if e >= L:  # lanes past the line (tiny lines): idle
                    continue
                a = (ln * lp + index(e)) * 2  # 8-byte elements, 4-byte words
                words += [a, a + 1]
            total += wavefronts(words)
    return total, len(patterns(L))


def test_swizzle_permutes_every_line():
    for m in (8, 16, 32, 64, 128, 256):
        assert sorted(fswz(i) for i in range(m)) == list(range(m))


def test_row_lines_need_the_minimum_wavefronts():
    for m in (16, 32, 64, 128, 256):
        got, insts = cost(m, fswz, pitch(m))
        assert got == 2 * insts, (m, got, insts)


def test_padding_it_replaced_was_conflicted():
    got, insts = cost(256, lambda i: i + (i >> 3), 256 + 32)
    assert got == 160 and insts == 48
