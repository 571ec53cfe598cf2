"""The 64 x 64 bit transpose the blocked run does with warp shuffles
(warp_transpose64 in the GPU library), restated lane by lane on the CPU: lane l
holds rows l and l + 32; the off-diagonal 32 x 32 blocks are swapped in each lane,
then both 32-bit halves are transposed at once by the recursive block swap (blocks
of 16, 8, 4, 2, 1, a shuffle with lane l ^ j per step).  Afterwards lane l holds
columns l and l + 32.  Checked against a direct transpose."""
import numpy as np

M64 = (1 << 64) - 1
MASKS = {16: 0x0000FFFF0000FFFF, 8: 0x00FF00FF00FF00FF, 4: 0x0F0F0F0F0F0F0F0F, 2: 0x3333333333333333,
         1: 0x5555555555555555}


def warp_transpose64(r0, r1):
    u0 = [(a & 0xFFFFFFFF) | ((b << 32) & M64) for a, b in zip(r0, r1)]
    u1 = [(a >> 32) | (b & 0xFFFFFFFF00000000) for a, b in zip(r0, r1)]
    for j in (16, 8, 4, 2, 1):
        m = MASKS[j]
        for u in (u0, u1):
            partner = [u[lane ^ j] for lane in range(32)]  # the shuffle
            out = []
            for lane in range(32):
                if lane & j == 0:
                    out.append(u[lane] ^ (((((u[lane] >> j) ^ partner[lane]) & m) << j) & M64))
                else:
                    out.append(u[lane] ^ (((partner[lane] >> j) ^ u[lane]) & m))
            u[:] = out
    return u0, u1


def test_shuffle_transpose_equals_direct_transpose():
    rng = np.random.default_rng(11)
    cases = [[0] * 64, [M64] * 64, [1 << i for i in range(64)]]
    for _ in range(40):
        cases.append([int(x) | (int(rng.integers(0, 2)) << 63) for x in rng.integers(0, 2**63, size=64, dtype=np.int64)])
    for rows in cases:
        c0, c1 = warp_transpose64(rows[:32], rows[32:])
        for c in range(64):
            want = sum(((rows[i] >> c) & 1) << i for i in range(64))
            assert (c0[c] if c < 32 else c1[c - 32]) == want, c
