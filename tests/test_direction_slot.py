"""The walks' direction slot (walk_device.cuh: dir_slot, morton_slot_direction) against
the reference's direction draw, state mod 6 (Walker/walker.h:566-582): the fold of the 64-bit state
keeps its residue mod 3, the product by the inverse of 3 mod 2^32 and the high product by 3 give
(-t) mod 3, and each slot stands for exactly one direction. CPU restatement of the device arithmetic."""
import numpy as np

INV3 = np.uint64(0xAAAAAAAB)
M32 = np.uint64(0xFFFFFFFF)


def fold(a):
    lo, hi = a & M32, a >> np.uint64(32)
    t = lo + hi
    return (t & M32) + (t >> np.uint64(32))  # the carry is worth 2^32 = 1 (mod 3); never overflows again


def slot(a):
    t = fold(a)
    m = (t * INV3) & M32
    s3 = (m * np.uint64(3)) >> np.uint64(32)
    return (np.uint64(2) * s3 + (a & np.uint64(1))).astype(np.int64)


def slot_direction(s):
    r3 = (3 - (s >> 1)) % 3
    return r3 + 3 * ((r3 ^ s) & 1)


def test_high_product_gives_minus_residue_mod_3():
    rng = np.random.default_rng(0)
    t = np.concatenate([rng.integers(0, 1 << 32, 2_000_000, dtype=np.uint64),
                        np.arange(0, 4096, dtype=np.uint64),
                        np.arange((1 << 32) - 4096, 1 << 32, dtype=np.uint64),
                        np.arange(0x55555550, 0x55555560, dtype=np.uint64),
                        np.arange(0xAAAAAAA0, 0xAAAAAAB0, dtype=np.uint64)])
    s3 = ((((t * INV3) & M32) * np.uint64(3)) >> np.uint64(32)).astype(np.int64)
    assert np.array_equal(s3, (-(t % np.uint64(3)).astype(np.int64)) % 3)


def test_slot_is_the_mod6_direction():
    rng = np.random.default_rng(1)
    a = rng.integers(0, np.iinfo(np.uint64).max, 2_000_000, dtype=np.uint64, endpoint=True)
    edges = np.array([0, 1, 5, 6, 2**64 - 1, 2**64 - 2, 2**63, 2**32 - 1, 2**32, 0xFFFFFFFF00000000], np.uint64)
    a = np.concatenate([a, edges])
    assert np.array_equal(slot_direction(slot(a)), (a % np.uint64(6)).astype(np.int64))


def test_slots_cover_each_direction_once():
    assert sorted(slot_direction(np.arange(6))) == [0, 1, 2, 3, 4, 5]


def test_bit_block_step_moves_by_slot():
    """walker_step's moves by slot (0:N(-y) 1:E(+x) 2:S(+y) 3:Down(-z) 4:Up(+z) 5:W(-x)) are the moves of the
    reference's directions (walker_defs.h: 0:N(-y) 1:W(-x) 2:S(+y) 3:E(+x) 4:Up(+z) 5:Down(-z))."""
    ref_move = {0: (0, -1, 0), 1: (-1, 0, 0), 2: (0, 1, 0), 3: (1, 0, 0), 4: (0, 0, 1), 5: (0, 0, -1)}
    for s in range(6):
        move = (int(s == 1) - int(s == 5), int(s == 2) - int(s == 0), int(s == 4) - int(s == 3))
        assert move == ref_move[int(slot_direction(np.array([s]))[0])], s
