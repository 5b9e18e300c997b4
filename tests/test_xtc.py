"""GROMACS .xtc trajectories (the reference's frame source, read through libxdrfile in
calcIR.cu:212-223, 341-395): the project's decoder and encoder, reached through
cir_traj_info / cir_traj_read / cir_xtc_write.  No .xtc file from GROMACS is available
here, so the decoder is checked against round trips and against streams built bit by bit
below from the format's description (independently of the C++ encoder)."""
import ctypes as C
import os
import struct

import numpy as np
import pytest

import calcir_gb300 as cg
from calcir_gb300._lib import CirError, check, load

RANGE = [0] * 9 + [8, 10, 12, 16, 20, 25, 32, 40, 50, 64, 80, 101, 128, 161, 203, 256, 322, 406, 512, 645, 812,
                   1024, 1290, 1625, 2048, 2580, 3250, 4096, 5060, 6501, 8192, 10321, 13003, 16384, 20642, 26007,
                   32768, 41285, 52015, 65536, 82570, 104031, 131072, 165140, 208063, 262144, 330280, 416127,
                   524287, 660561, 832255, 1048576, 1321122, 1664510, 2097152, 2642245, 3329021, 4194304, 5284491,
                   6658042, 8388607, 10568983, 13316085, 16777216]


def _write(path, xyz, box, times, prec=1000.0):
    lib = load()
    xyz = np.ascontiguousarray(xyz, np.float32)
    b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, np.float32), (xyz.shape[0], 3)))
    t = np.ascontiguousarray(times, np.float32)
    check(lib.cir_xtc_write(str(path).encode(), xyz.shape[1], xyz.shape[0], C.c_void_p(xyz.ctypes.data),
                            C.c_void_p(b.ctypes.data), C.c_void_p(t.ctypes.data), C.c_float(prec)))


def _info(path):
    na, nf, dt = C.c_int(), C.c_int(), C.c_float()
    check(load().cir_traj_info(str(path).encode(), C.byref(na), C.byref(nf), C.byref(dt)))
    return na.value, nf.value, dt.value


def _read(path, first, count, natoms):
    xyz = np.zeros((count, natoms, 3), np.float32)
    box = np.zeros((count, 3), np.float32)
    t = np.zeros(count, np.float32)
    check(load().cir_traj_read(str(path).encode(), first, count, C.c_void_p(xyz.ctypes.data),
                               C.c_void_p(box.ctypes.data), C.c_void_p(t.ctypes.data)))
    return xyz, box, t


def test_round_trip_water(tmp_path):
    xyz, box = cg.synth_trajectory(128, 7, seed=5)
    times = 0.010 * np.arange(7) + 1e-7 * np.arange(7)          # the spacing is rounded to the precision
    path = tmp_path / "w.xtc"
    _write(path, xyz, box, times)
    assert os.path.getsize(path) < xyz.nbytes / 2                # compressed
    na, nf, dt = _info(path)
    assert (na, nf) == (xyz.shape[1], 7) and dt == pytest.approx(0.010, abs=1e-7)
    out, ob, ot = _read(path, 0, 7, na)
    assert np.abs(out - xyz).max() <= 0.5e-3 + 1e-6
    np.testing.assert_array_equal(ob, np.broadcast_to(box, (7, 3)))
    np.testing.assert_array_equal(ot, times.astype(np.float32))
    one, _, t1 = _read(path, 4, 1, na)                           # random access
    np.testing.assert_array_equal(one[0], out[4])
    assert t1[0] == ot[4]


def test_quantisation_is_round_half_away_from_zero(tmp_path):
    pos = np.array([[0.0004, -0.0004, 0.0015], [-0.0015, 0.0025, -0.0025]] * 6, np.float32)[None]
    pos = pos + np.array([1.0, 1.0, 1.0], np.float32)            # keep the values exact in float
    path = tmp_path / "q.xtc"
    _write(path, pos, [3, 3, 3], [0.0])
    out, _, _ = _read(path, 0, 1, pos.shape[1])
    expect = np.sign(pos * 1000) * np.floor(np.abs(pos * 1000) + 0.5) / np.float32(1000)
    np.testing.assert_allclose(out, expect, atol=2e-7)


def test_few_atoms_are_stored_uncompressed(tmp_path):
    rng = np.random.default_rng(1)
    pos = rng.uniform(0, 3, (3, 9, 3)).astype(np.float32)
    path = tmp_path / "s.xtc"
    _write(path, pos, [3, 3, 3], [0.0, 0.5, 1.0])
    out, _, _ = _read(path, 0, 3, 9)
    np.testing.assert_array_equal(out, pos)


def test_huge_range_uses_per_axis_fields(tmp_path):
    rng = np.random.default_rng(2)
    pos = rng.uniform(0, 40, (2, 50, 3)).astype(np.float32)     # 40 nm at 1e6 per nm: > 2^24 per axis
    path = tmp_path / "h.xtc"
    _write(path, pos, [40, 40, 40], [0.0, 1.0], prec=1e6)
    out, _, _ = _read(path, 0, 2, 50)
    assert np.abs(out - pos).max() <= 0.5e-6 + 4e-6


class _Bits:
    """MSB-first bit stream, as the format reads it."""

    def __init__(self):
        self.bits = []

    def put(self, v, n):
        self.bits += [(v >> (n - 1 - i)) & 1 for i in range(n)]

    def triple(self, nbits, sizes, c):
        v = (c[0] * sizes[1] + c[1]) * sizes[2] + c[2]
        while nbits > 8:                                        # low bytes first, then the top bits
            self.put(v & 0xFF, 8)
            v >>= 8
            nbits -= 8
        if nbits > 0:
            self.put(v, nbits)

    def bytes(self):
        b = self.bits + [0] * (-len(self.bits) % 8)
        return bytes(int("".join(map(str, b[i:i + 8])), 2) for i in range(0, len(b), 8))


def _triple_bits(sizes):
    p = sizes[0] * sizes[1] * sizes[2]
    nbytes = 0
    while p >> 8:
        p >>= 8
        nbytes += 1
    b = 0
    while p >= (1 << b):
        b += 1
    return b + 8 * nbytes


def test_decoder_known_answer_stream(tmp_path):
    """A 12-atom frame written bit by bit: runs of two small atoms (first one swapped before
    the large atom), a repeated run (flag 0), the small index stepping down and up again."""
    prec = 1000.0
    big = {1: (500, 600, 700), 4: (900, 300, 250), 7: (100, 800, 400), 8: (950, 950, 50), 10: (10, 20, 30)}
    coords = {}
    minint, maxint = [0, 0, 0], [1000, 1000, 1000]
    sizes = [maxint[d] - minint[d] + 1 for d in range(3)]
    nbits = _triple_bits(sizes)
    bs = _Bits()
    idx = 15                                                    # small range 32, offset 16

    def small(ref, delta, sidx):
        half = RANGE[sidx] // 2
        bs.triple(sidx, [RANGE[sidx]] * 3, [delta[d] + half for d in range(3)])
        return tuple(ref[d] + delta[d] for d in range(3))

    # large atom 1, run of 2 small atoms: atom 0 (relative to 1), atom 2 (relative to 0)
    bs.triple(nbits, sizes, [big[1][d] - minint[d] for d in range(3)])
    bs.put(1, 1); bs.put(3 * 2 + 1, 5)                          # run 6, small index unchanged
    coords[1] = big[1]
    coords[0] = small(big[1], (-5, 3, 15), idx)
    coords[2] = small(coords[0], (7, -16, 0), idx)
    # large atom 4, the same run again (flag 0): atoms 3 and 5
    bs.triple(nbits, sizes, [big[4][d] - minint[d] for d in range(3)])
    bs.put(0, 1)
    coords[4] = big[4]
    coords[3] = small(big[4], (1, 1, -1), idx)
    coords[5] = small(coords[3], (15, -15, 2), idx)
    # large atom 7, run of one small atom (atom 6), then the small index steps down
    bs.triple(nbits, sizes, [big[7][d] - minint[d] for d in range(3)])
    bs.put(1, 1); bs.put(3 * 1 + 0, 5)                          # run 3, small index - 1
    coords[7] = big[7]
    coords[6] = small(big[7], (-16, 0, 9), idx)
    idx -= 1
    # large atom 8 alone, the small index steps up
    bs.triple(nbits, sizes, [big[8][d] - minint[d] for d in range(3)])
    bs.put(1, 1); bs.put(0 + 2, 5)                              # run 0, small index + 1
    coords[8] = big[8]
    idx += 1
    # large atom 10 with atoms 9 and 11
    bs.triple(nbits, sizes, [big[10][d] - minint[d] for d in range(3)])
    bs.put(1, 1); bs.put(3 * 2 + 1, 5)
    coords[10] = big[10]
    coords[9] = small(big[10], (2, 2, 2), idx)
    coords[11] = small(coords[9], (-3, 4, -5), idx)
    payload = bs.bytes()
    frame = struct.pack(">iiif", 1995, 12, 0, 0.0) + struct.pack(">9f", 2, 0, 0, 0, 2, 0, 0, 0, 2)
    frame += struct.pack(">if", 12, prec) + struct.pack(">3i", *minint) + struct.pack(">3i", *maxint)
    frame += struct.pack(">ii", 15, len(payload)) + payload + b"\0" * (-len(payload) % 4)
    path = tmp_path / "k.xtc"
    path.write_bytes(frame)
    out, box, _ = _read(path, 0, 1, 12)
    expect = np.array([coords[i] for i in range(12)], np.float32) * np.float32(1.0 / prec)
    np.testing.assert_array_equal(out[0], expect)
    np.testing.assert_array_equal(box[0], [2, 2, 2])


def test_malformed_files_are_reported(tmp_path):
    xyz, box = cg.synth_trajectory(64, 3, seed=6)
    path = tmp_path / "m.xtc"
    _write(path, xyz, box, [0.0, 0.01, 0.02])
    data = path.read_bytes()
    bad = tmp_path / "cut.xtc"
    bad.write_bytes(data[:len(data) - 37])                      # the last frame is cut
    with pytest.raises(CirError):
        _info(bad)
    bad.write_bytes(data[:40])
    with pytest.raises(CirError):
        _info(bad)
