"""Pin the oracle's Morton key operations to the reference's own key tests.

Every case re-expresses a TEST of test/map/keyops/keyops_unittest.cpp (supereight2) with the
same inputs and expected values; the reference's helper adapt_to_scale (:33-40) is restated as
``adapt``.
"""
import numpy as np
import pytest


def adapt(c, s):
    return tuple((v >> s) << s for v in c)


def enc_key(o, c, s):
    import ctypes
    k = ctypes.c_uint64()
    full = o.lib().so_encode_key(int(c[0]), int(c[1]), int(c[2]), int(s), ctypes.byref(k))
    return k.value, bool(full)


def dec_key(o, key):
    import ctypes
    c = np.zeros(3, np.int32)
    s = ctypes.c_uint64()
    o.lib().so_decode_key(int(key), c, ctypes.byref(s))
    return tuple(int(v) for v in c), s.value


def test_encode_decode_code(oracle):
    # keyops_unittest.cpp:14-30
    L = oracle.lib()
    c = np.zeros(3, np.int32)
    for x in range(513, 1028, 19):
        for y in range(254, 844, 13):
            for z in range(0, 553, 11):
                code = L.so_encode_code(x, y, z)
                L.so_decode_code(code, c)
                assert tuple(c) == (x, y, z)


def test_encode_decode_key(oracle):
    # keyops_unittest.cpp:42-78
    for x in range(513, 1028, 11):
        for y in range(254, 844, 19):
            for z in range(0, 553, 23):
                for s in range(5):
                    key, _ = enc_key(oracle, (x, y, z), s)
                    c, sc = dec_key(oracle, key)
                    assert c == adapt((x, y, z), s) and sc == s
    assert enc_key(oracle, (333, 222, 111), 4)[1] is False
    assert enc_key(oracle, (332, 220, 108), 2)[1] is True


def test_code_to_child_idx(oracle):
    # keyops_unittest.cpp:80-98
    L = oracle.lib()
    coord = np.zeros(3, np.int64)
    for s in range(8):
        coord += (1 << s) * np.array([(s & 1) > 0, (s & 2) > 0, (s & 4) > 0])
    code = L.so_encode_code(*[int(v) for v in coord])
    for s in range(8):
        assert L.so_code_to_child_idx(code, s) == s


def test_key_to_code_scale(oracle):
    # keyops_unittest.cpp:100-126
    L = oracle.lib()
    c = np.zeros(3, np.int32)
    for x in range(513, 1028, 13):
        for y in range(254, 844, 7):
            for z in range(0, 553, 29):
                for s in range(5):
                    key, _ = enc_key(oracle, (x, y, z), s)
                    code, scale = key >> 5, key & 0x1F
                    L.so_decode_code(code, c)
                    assert tuple(c) == adapt((x, y, z), s) and scale == s


def test_key_at_scale_and_parent(oracle):
    # keyops_unittest.cpp:128-158 (KeyAtScale), :160-176 (CodeAtScale), :178-190 (ParentKey)
    import ctypes
    L = oracle.lib()
    base, _ = enc_key(oracle, (170, 204, 240), 0)
    parent = L.so_parent_key(base)
    out = ctypes.c_uint64()
    for s in range(1, 8):
        L.so_key_at_scale(base, s, ctypes.byref(out))
        assert out.value == parent
        L.so_code_at_scale(base, s, ctypes.byref(out))
        assert out.value == parent >> 5
        parent = L.so_parent_key(parent)
    base, _ = enc_key(oracle, (160, 192, 240), 4)
    for s in range(8):
        assert bool(L.so_key_at_scale(base, s, ctypes.byref(out))) == (s >= 4)
    for s in range(7):
        child, _ = enc_key(oracle, (170, 204, 240), s)
        ought, _ = enc_key(oracle, (170, 204, 240), s + 1)
        assert L.so_parent_key(child) == ought


def test_block_key_and_code(oracle):
    # keyops_unittest.cpp:192-218
    L = oracle.lib()
    base = 0x1FFFFFFFFFFFFE0
    ought = [0x1FFFFFFFFFFFFE0, 0x1FFFFFFFFFFFF00, 0x1FFFFFFFFFFF800, 0x1FFFFFFFFFFC000]
    for s in range(4):
        assert L.so_block_key(base, s) == ought[s]
        assert L.so_block_code(base, s) == ought[s] >> 5


def test_is_child_is_sibling(oracle):
    # keyops_unittest.cpp:220-271
    import ctypes
    L = oracle.lib()
    base, _ = enc_key(oracle, (170, 204, 240), 0)
    pk, ck = ctypes.c_uint64(), ctypes.c_uint64()
    for p in range(1, 7):
        for c in range(7):
            L.so_key_at_scale(base, p, ctypes.byref(pk))
            L.so_key_at_scale(base, c, ctypes.byref(ck))
            assert bool(L.so_is_child(pk.value, ck.value)) == (c < p)
    for s in range(7):
        pc = adapt((170, 204, 240), s + 1)
        parent, _ = enc_key(oracle, pc, s + 1)
        kids = []
        for i in range(8):
            cc = tuple(pc[a] + (1 << s) * ((i >> a) & 1) for a in range(3))
            kids.append(enc_key(oracle, cc, s)[0])
        for a in kids:
            for b in kids:
                assert L.so_is_siblings(a, b)
            assert not L.so_is_siblings(parent, a)


COORDS_UNIQUE = [(56, 12, 12), (56, 12, 12), (128, 128, 128), (128, 132, 130), (128, 132, 130),
                 (300, 21, 829), (628, 36, 227), (436, 18, 436), (128, 241, 136), (128, 241, 136)]
SCALES_UNIQUE = [0, 0, 1, 0, 1, 3, 4, 2, 3, 3]


def _keys(oracle, coords, scales):
    return np.array([enc_key(oracle, c, s)[0] for c, s in zip(coords, scales)], np.uint64)


def test_unique_keys_and_codes(oracle):
    # keyops_unittest.cpp:273-312 (UniqueKeys), :314-368 (UniqueCodes)
    L = oracle.lib()
    keys = _keys(oracle, COORDS_UNIQUE, SCALES_UNIQUE)
    out = np.zeros(16, np.uint64)
    n = L.so_unique_keys(keys.copy(), len(keys), out)
    assert n == 8 and len(set(out[:n].tolist())) == 8
    n = L.so_unique_codes(keys.copy(), len(keys), out)
    assert n == 7 and len(set(out[:n].tolist())) == 7
    assert enc_key(oracle, (128, 132, 130), 0)[0] in out[:n].tolist()


def test_unique_allocation(oracle):
    # keyops_unittest.cpp:370-427
    L = oracle.lib()
    coords = [(0, 0, 0), (32, 16, 32), (40, 24, 32), (128, 128, 128), (144, 128, 160),
              (144, 132, 164), (512, 512, 1024), (512, 544, 1056), (512, 545, 1056),
              (512, 544, 1056)]
    scales = [6, 5, 3, 7, 4, 2, 6, 4, 1, 1]
    keys = _keys(oracle, coords, scales)
    out = np.zeros(16, np.uint64)
    n = L.so_unique_allocation(keys, len(keys), 2, out)
    ought = _keys(oracle, [(40, 24, 32), (144, 132, 164), (512, 545, 1056), (512, 544, 1056)],
                  [3, 2, 1, 1])
    _assert_like_reference(out[:n], ought)


def _assert_like_reference(unique, ought):
    # The reference asserts the count, pairwise distinct neighbours, and membership; its
    # membership loop never resets `contains`, so only ought[0] is effectively checked
    # (keyops_unittest.cpp:413-427). The later expected entries are not what the function
    # produces (block_key keeps the key's own scale), so they are not asserted here either.
    assert len(unique) == len(ought)
    assert all(unique[i - 1] != unique[i] for i in range(1, len(unique)))
    assert int(ought[0]) in unique.tolist()


def test_unique_at_scale(oracle):
    # keyops_unittest.cpp:429-480
    L = oracle.lib()
    coords = [(0, 0, 0), (32, 16, 32), (40, 24, 32), (128, 128, 128), (144, 128, 160),
              (144, 132, 164), (512, 512, 1024), (512, 544, 1056), (512, 545, 1056),
              (513, 545, 1056)]
    scales = [6, 5, 3, 6, 4, 2, 6, 4, 1, 1]
    keys = np.sort(_keys(oracle, coords, scales))
    out = np.zeros(16, np.uint64)
    n = L.so_unique_at_scale(keys, len(keys), 5, out)
    ought = _keys(oracle, [(32, 0, 32), (128, 128, 160), (512, 512, 1024)], [5, 5, 5])
    _assert_like_reference(out[:n], ought)
    # keyops_unittest.cpp:505-540: the same keys at scale 3
    n = L.so_unique_at_scale(keys, len(keys), 3, out)
    ought = _keys(oracle, [(40, 24, 32), (144, 128, 160), (512, 544, 1056)], [3, 3, 3])
    assert n == 3
    assert sorted(out[:n].tolist()) == sorted(ought.tolist())


@pytest.mark.parametrize("v", [0, 1, 2, 0x7FFFF, 0x5A5A5, 12345])
def test_expand_compact_roundtrip(oracle, v):
    L = oracle.lib()
    assert L.so_compact(L.so_expand(v)) == v
