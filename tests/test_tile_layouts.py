"""Index arithmetic of the TMA-fed and fused kernels' shared-memory layouts,
restated and checked on the CPU (no GPU, no library call).

Each check restates a kernel's own formulas (named below) and verifies:
* every staged element is written once and read back from where the next
  stage (the MMA or the FMA loop) expects it;
* the accesses of one warp instruction spread over the banks as the
  kernels' comments claim.

Shared memory is modelled as 32 banks of 4 bytes. A warp's 16-byte access
needs at least 4 wavefronts (512 bytes), so for those the check counts
distinct 16-byte bank groups per quarter of the warp's data. TMA's 128-byte
swizzle is modelled as the 16-byte chunk q of a box row r landing at chunk
q ^ (r % 8) of that row. That is the pattern the MMA's 128-byte swizzled
layout uses too; the GPU parity tests check it for real.
"""
import numpy as np


def swz128(row, chunk):
    """Byte offset of 16-byte chunk `chunk` of 128-byte row `row` in a
    1024-byte-aligned 128-byte-swizzled tile."""
    return row * 128 + ((chunk ^ (row % 8)) << 4)


def banks_of_words(word_addrs):
    return np.asarray(word_addrs) % 32


def test_nn_update_rewrite_places_every_element_for_the_mma():
    """tc_nn_tma_kernel: A1's 128 x 32 stage arrives as four 32 x 32 boxes
    (rows inner), element (r, k) at box r/32, row k, chunk (r%32)/4, word
    r%4.  Warp w (of 8) takes row groups 4w..4w+3; lane l takes K index l.
    The rewrite writes (r, k) to the K-major tile at row r, chunk k/4, word
    k%4, which is where the MMA's descriptor reads it."""
    A = np.arange(128 * 32).reshape(128, 32)  # distinct tags
    raw = np.full(4096, -1)
    for r in range(128):
        for k in range(32):
            off = (r // 32) * 4096 + swz128(k, (r % 32) // 4) + (r % 4) * 4
            raw[off // 4] = A[r, k]
    assert (raw >= 0).all()
    out = np.full(4096, -1)
    for warp in range(8):
        for i in range(4):
            g = warp * 4 + i
            r = 4 * g
            lanes = np.arange(32)
            k = lanes
            src = (r >> 5) * 4096 + k * 128 + ((((r & 31) >> 2) ^ (k & 7)) << 4)
            # one 16-byte read per lane: 32 x 16 B = 4 wavefronts at best
            for q in range(4):
                rr = r + q
                dst = rr * 128 + (((k >> 2) ^ (rr & 7)) << 4) + (k & 3) * 4
                # one 4-byte store per lane: 32 distinct banks
                assert len(set(banks_of_words(dst // 4))) == 32
                assert (out[dst // 4] == -1).all()
                out[dst // 4] = raw[(src + 4 * q) // 4]
    for r in range(128):
        for k in range(32):
            assert out[(swz128(r, k // 4) + (k % 4) * 4) // 4] == A[r, k]


def test_tn_projection_reads_hit_distinct_bank_groups():
    """gemm_tn_tma: a 64-row step arrives as 32 x 32 boxes (rows inner);
    thread (ig, jg) of a K slice reads rows k4*4.. of columns ig + 8u (A)
    and jg + 8v (B) as 16-byte chunks at chunk k4 ^ (column % 8).  Within a
    warp (lt = 0..31: ig = lt % 8, jg = lt / 8) the A reads touch 8
    distinct 16-byte groups and the B reads 4, so each is one wavefront."""
    for k4 in range(8):
        for u in range(4):
            lt = np.arange(32)
            ig, jg = lt & 7, lt >> 3
            a_off = (ig + 8 * u) * 128 + ((k4 ^ ig) << 4)
            b_off = (jg + 8 * u) * 128 + ((k4 ^ jg) << 4)
            assert len(set((a_off // 16) % 8)) == 8
            assert len(set(a_off)) == 8
            assert len(set((b_off // 16) % 8)) == 4
            assert len(set(b_off)) == 4


def test_tn_projection_slices_cover_the_tile_once():
    """gemm_tn_tma / gemm_tn_fused epilogue: four K slices of 64 threads,
    thread (ig, jg) owning outputs (ig + 8u, jg + 8v) (TMA form) or
    (4 ig + u, 4 jg + v) (register form); each 32 x 32 output is owned once
    per slice."""
    for form in ("tma", "fused"):
        own = np.zeros((32, 32), int)
        for lt in range(64):
            ig, jg = (lt & 7, lt >> 3) if form == "tma" else (lt >> 3, lt & 7)
            for u in range(4):
                for v in range(4):
                    i, j = (ig + 8 * u, jg + 8 * v) if form == "tma" else (4 * ig + u, 4 * jg + v)
                    own[i, j] += 1
        assert (own == 1).all()


def test_fused_projection_staging_is_conflict_free_and_complete():
    """gemm_tn_fused (register-staged form): slot e of thread (warp, lane)
    holds rows 4kq..4kq+3 of step column gc = 4 (2 warp + e/2) + lane/8,
    kq = 8 (e%2) + lane%8, stored at [4kq + q][((gc%32)/4 ^ kq%8) * 4 +
    gc%4].  Each of the 4 store instructions of a warp hits 32 banks, and
    every (row, column) of the 64 x 64 step is written once."""
    seen = np.zeros((2, 64, 32), int)
    for warp in range(8):
        for e in range(4):
            for q in range(4):
                lane = np.arange(32)
                kq = 8 * (e & 1) + (lane & 7)
                gc = 4 * (warp * 2 + (e >> 1)) + (lane >> 3)
                col = ((((gc & 31) >> 2) ^ (kq & 7)) << 2) + (gc & 3)
                row = 4 * kq + q
                word = row * 32 + col
                assert len(set(banks_of_words(word))) == 32
                for l in range(32):
                    seen[int(gc[l] >= 32), row[l], col[l]] += 1
    assert (seen == 1).all()


def test_nn_fused_loader_and_compute_cover_the_block():
    """gemm_nn_fused: the A1 chunk loader (float4 slot e of thread t: column
    (t + 256 e) / 32 of the chunk, rows 4 ((t + 256 e) % 32)..) writes each
    of the 128 x 32 elements once; the compute mapping (rows 4 rg.., columns
    4 cg.., rg = 8 (w % 4) + l % 8, cg = 4 (w / 4) + l / 8) owns each of
    the 128 x 32 outputs once."""
    seen = np.zeros((32, 128), int)
    for t in range(256):
        for e in range(4):
            idx = t + 256 * e
            kk, r4 = idx >> 5, idx & 31
            seen[kk, 4 * r4:4 * r4 + 4] += 1
    assert (seen == 1).all()
    own = np.zeros((128, 32), int)
    for t in range(256):
        w, l = t >> 5, t & 31
        rg, cg = (w & 3) * 8 + (l & 7), (w >> 2) * 4 + (l >> 3)
        own[4 * rg:4 * rg + 4, 4 * cg:4 * cg + 4] += 1
    assert (own == 1).all()
