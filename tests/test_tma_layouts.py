"""CPU checks of the shared-memory index arithmetic of the tensor-core product
(`tc_bgemm_kernel` in bn_dense.cuh), restated in Python: the 128-byte swizzle the
TMA boxes land in (16-byte chunk c of row r at chunk c ^ (r % 8)), the transposing
split of an M/N-major operand into the K-major layout the MMAs read, and the lane
pattern it uses (block (box j, k chunk a, M/N chunk c) with a = c ^ d), which is
meant to give every eight lanes eight distinct 16-byte bank groups on both the
reads and the writes.  The kernel's numbers against float64 are in
tests/test_gpu_dense.py."""
import numpy as np


def raw_offset(j, k, mn):
    """byte offset of element (K row k, M/N column 32 j + mn) in the raw boxes"""
    return j * 4096 + k * 128 + (((mn >> 2) ^ (k & 7)) << 4) + (mn & 3) * 4


def kmajor_offset(n, k):
    """byte offset of element (row n, K column k) in the K-major swizzled operand"""
    return n * 128 + (((k >> 2) ^ (n & 7)) << 4) + (k & 3) * 4


def split_blocks(rows, nbox, threads=256):
    """(thread, block) pairs of the transposing split, as the kernel walks them"""
    for t in range(threads):
        for blk in range(t, 64 * nbox, threads):
            j, d, c = blk >> 6, (blk >> 3) & 7, blk & 7
            a = c ^ d
            if 32 * j + 4 * c >= rows:
                continue
            yield t, j, a, c


def test_swizzle_offsets_are_a_permutation():
    offs = {raw_offset(j, k, mn) for j in range(4) for k in range(32) for mn in range(32)}
    assert offs == set(range(0, 4 * 4096, 4))
    offs = {kmajor_offset(n, k) for n in range(112) for k in range(32)}
    assert offs == set(range(0, 112 * 128, 4))


def test_transposing_split_moves_every_element_once():
    for rows, nbox in ((128, 4), (112, 4), (208, 7)):
        src = np.arange(nbox * 32 * 32, dtype=np.int64)  # value = raw word index
        raw = np.full(nbox * 1024, -1, dtype=np.int64)
        for j in range(nbox):
            for k in range(32):
                for mn in range(32):
                    raw[raw_offset(j, k, mn) // 4] = src[(j * 32 + k) * 32 + mn]
        hi = np.full(rows * 32, -1, dtype=np.int64)
        for _, j, a, c in split_blocks(rows, nbox):
            for q in range(4):  # the four K rows 4a + q
                k = 4 * a + q
                for p in range(4):  # the four M/N columns 4c + p
                    n = 32 * j + 4 * c + p
                    hi[kmajor_offset(n, k) // 4] = raw[raw_offset(j, k, 4 * c + p) // 4]
        assert (hi >= 0).all()
        for n in range(rows):
            for k in range(32):
                j, mn = divmod(n, 32)
                assert hi[kmajor_offset(n, k) // 4] == (j * 32 + k) * 32 + mn


def test_split_lane_pattern_hits_distinct_bank_groups():
    """For each warp instruction of the split (one 16-byte load of row 4a + q, or
    one 16-byte store of row 32 j + 4 c + p), each group of eight lanes covers eight
    distinct 16-byte bank groups (address bits 4-6), so 32 lanes take the minimum
    four wavefronts."""
    blocks = list(split_blocks(128, 4))
    by_thread = {}
    for t, j, a, c in blocks:
        by_thread.setdefault(t, []).append((j, a, c))
    for it in range(2):  # each thread's first and second block
        for w in range(8):
            for g in range(4):
                lanes = [32 * w + 8 * g + i for i in range(8)]
                work = [by_thread[t][it] for t in lanes if len(by_thread.get(t, [])) > it]
                if len(work) < 8:
                    continue
                for q in range(4):
                    groups = {(raw_offset(j, 4 * a + q, 4 * c) >> 4) & 7 for j, a, c in work}
                    assert len(groups) == 8
                for p in range(4):
                    groups = {(kmajor_offset(32 * j + 4 * c + p, 4 * a) >> 4) & 7 for j, a, c in work}
                    assert len(groups) == 8
