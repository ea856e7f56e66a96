"""Index arithmetic of the shared-memory table lookups (CPU): every lookup
visits each byte position once with its own byte, and at every step eight
consecutive threads read eight distinct bank groups (a 16-byte slot's bank
group is its index mod 8), which is what makes the random lookups
conflict-free. The formulas restate those of csrc/gf_tab.cuh (gf_mul_tab and
the byte-table rows of gf_tab_row_direct),
csrc/open.cu (combined basis), csrc/zerocheck.cu (round-1 extension tables,
phi8 nibble tables, skip tables) and csrc/lincheck.cu (stripe fold)."""


def byte_perm(x, y, s):
    """__byte_perm(x, y, s): result byte i = byte (s >> 4i) & 7 of {y:x}."""
    b = [(x >> (8 * i)) & 255 for i in range(4)] + [(y >> (8 * i)) & 255 for i in range(4)]
    return sum(b[(s >> (4 * i)) & 7] << (8 * i) for i in range(4))


def gf_tab_offsets(y_bytes, lane):
    """Byte offsets into the 64 KiB byte tables that gf_mul_tab reads, in step order."""
    w = [sum(y_bytes[4 * j + i] << (8 * i) for i in range(4)) for j in range(4)]
    rot = lane & 7
    sw = bool(rot & 4)
    yp = [w[1], w[0], w[3], w[2]] if sw else list(w)
    perm = [0x3210, 0x2301, 0x1032, 0x0123][rot & 3]
    yp = [byte_perm(v, 0, perm) for v in yp]
    xk = rot << 4
    out = []
    for st in range(16):
        vb = byte_perm(yp[st >> 2], 0, 0x4404 | ((st & 3) << 4))
        out.append((vb | (st << 4)) ^ xk)
    return out


def test_gf_tab_visits_each_position_with_its_byte():
    y = list(range(100, 116))  # byte k of y = 100 + k
    for lane in range(32):
        offs = gf_tab_offsets(y, lane)
        slots = [o >> 4 for o in offs]
        pos = sorted(s & 15 for s in slots)
        assert pos == list(range(16)), lane
        for s in slots:
            assert s >> 4 == y[s & 15], (lane, s)  # table row = byte of that position


def test_gf_tab_bank_groups_distinct():
    y = [7] * 16  # worst case for value-dependent layouts: all bytes equal
    for st in range(16):
        for l0 in range(0, 32, 8):
            groups = {(gf_tab_offsets(y, l)[st] >> 4) % 8 for l in range(l0, l0 + 8)}
            assert len(groups) == 8, (st, l0)


def test_combined_basis_rotation():
    # lane rotation rot = thread & 15 visits q = (rot + t) & 15; slot (v << 4) + q
    for t in range(16):
        for l0 in range(0, 32, 8):
            groups = {(((9 << 4) + ((l & 15) + t & 15)) % 8) for l in range(l0, l0 + 8)}
            assert len(groups) == 8
    for rot in range(16):
        assert sorted((rot + t) & 15 for t in range(16)) == list(range(16))


def test_zc_round1_extension_and_phi_layouts():
    # extension table: entry (q, v, c) at slot ((q * 256 + v) << 3) + c, lane l reads c = (l + k) & 7
    for k in range(8):
        for l0 in range(0, 32, 8):
            groups = {(((3 * 256 + 200) << 3) + ((l + k) & 7)) % 8 for l in range(l0, l0 + 8)}
            assert len(groups) == 8
    # eq-weighted phi8 nibble tables: L[j] of replica r at slot 4 j + r, H[g]
    # at 64 + 4 g + r, lane l reads replica l & 3; every (table, entry,
    # replica) has its own slot and a quarter warp puts at most two lanes in
    # one bank group for any nibbles it reads
    slots = {4 * j + r for j in range(16) for r in range(4)} | {64 + 4 * j + r for j in range(16) for r in range(4)}
    assert slots == set(range(128))
    import random
    rng = random.Random(3)
    for _ in range(200):
        nib = [rng.randrange(16) for _ in range(8)]
        groups = [(64 + 4 * nib[l] + (l & 3)) % 8 for l in range(8)]
        assert max(groups.count(g) for g in groups) <= 2
    # skip-fold tables of the grouped round 0: entry (v, c) at slot (v << 3) + c
    for k in range(8):
        assert len({((33 << 3) + ((l & 7) + k & 7)) % 8 for l in range(8)}) == 8


def test_lincheck_stripe_rotation():
    # t8[v][q] at slot v * 8 + q, lane reads stripe q = (lane8 + st) & 7
    for st in range(8):
        assert len({(5 * 8 + ((l + st) & 7)) % 8 for l in range(8)}) == 8
    for l in range(8):
        assert sorted((l + st) & 7 for st in range(8)) == list(range(8))


def test_phi8_table_weights_by_eq():
    # zc_round1_kernel's per-warp table T8[v] = phi8(v) e: lane l writes slots
    # l + 32 i (i < 8) as the XOR of phi8(2^k) e over the bits k < 5 of l and,
    # along a Gray walk over g (i = g ^ (g >> 1), one XOR of basis 5 + ctz(g)
    # per step), over the bits k of i at 5 + k; every slot once, and a quarter
    # warp's eight stores are 128 consecutive bytes
    import oracle_lib as O
    e = (0x0123456789ABCDEF, 0xF0E1D2C3B4A59687)
    P = [O.gf_mul(O.phi8(1 << k), e) for k in range(8)]

    def xor(a, b):
        return (a[0] ^ b[0], a[1] ^ b[1])
    t8 = {}
    for lane in range(32):
        lo = (0, 0)
        for k in range(5):
            if (lane >> k) & 1:
                lo = xor(lo, P[k])
        hp = (0, 0)
        for g in range(8):
            if g:
                hp = xor(hp, P[5 + (0 if g & 1 else 1 if g & 2 else 2)])
            i = g ^ (g >> 1)
            slot = lane + 32 * i
            assert slot not in t8
            t8[slot] = xor(lo, hp)
    assert sorted(t8) == list(range(256))
    for v in range(256):
        assert t8[v] == O.gf_mul(O.phi8(v), e), v
    for g in range(8):  # the slots a quarter warp writes at one step
        i = g ^ (g >> 1)
        for q in range(4):
            slots = [lane + 32 * i for lane in range(8 * q, 8 * q + 8)]
            assert slots == list(range(slots[0], slots[0] + 8)) and slots[0] % 8 == 0


def test_gf_tab_row_direct_gray_walk():
    # gf_tab_row_direct: slot of step jj is (g << 8) + (j << 4) + k with j = jj ^ (jj >> 1),
    # reached from the previous step by one XOR of image ctz(jj); all 4096 slots once
    def ctz4(j):
        return 0 if j & 1 else 1 if j & 2 else 2 if j & 4 else 3
    written = []
    for item in range(256):
        g, k = item >> 4, item & 15
        prev = 0
        for jj in range(16):
            j = jj ^ (jj >> 1)
            if jj:
                assert prev ^ j == 1 << ctz4(jj)  # the Gray step flips bit ctz(jj) of j
            prev = j
            slot = (g << 8) + (j << 4) + k
            assert slot == ((16 * g + j) << 4) + k
            written.append(slot)
    assert sorted(written) == list(range(4096))
    for base in range(0, 256, 8):  # eight consecutive items: distinct bank groups at every step
        for jj in range(16):
            j = jj ^ (jj >> 1)
            assert len({(((base + q) >> 4 << 8) + (j << 4) + ((base + q) & 15)) % 8 for q in range(8)}) == 8


def test_gf_tab_row_direct_values():
    # the row formula: t v x^(8k) = sum_{bits b of j} t x^(8k+b) + sum_{bits b of g} t x^(8k+4+b), v = 16 g + j
    import oracle_lib as O
    t = (0x243F6A8885A308D3, 0x13198A2E03707344)

    def xpow(i):
        return (1 << i, 0) if i < 64 else (0, 1 << (i - 64))

    for k in (0, 5, 15):
        B = [O.gf_mul(t, xpow(8 * k + b)) for b in range(8)]
        for v in (0, 1, 0x5A, 0xFF, 0x80):
            g, j = v >> 4, v & 15
            acc = (0, 0)
            for b in range(4):
                if (j >> b) & 1:
                    acc = (acc[0] ^ B[b][0], acc[1] ^ B[b][1])
                if (g >> b) & 1:
                    acc = (acc[0] ^ B[4 + b][0], acc[1] ^ B[4 + b][1])
            want = O.gf_mul(t, O.gf_mul((v, 0), xpow(8 * k)))
            assert acc == want, (k, v)


def test_zc_round1_eq_weight_factors():
    # round 1 multiplies each row by f0(par) f1(xs2) (compile-time constants)
    # and the block's sum by f2(h): e8(xs) = prod_v (bit v of xs ? C_v : 1 + C_v)
    # with xs = 4 h + 2 xs2 + par, C = (0xF7, 0x53, 0xB5)
    import oracle_lib as O
    mul = O.lib().oracle_gf8_mul
    C = (0xF7, 0x53, 0xB5)

    def f(v, bit):
        return C[v] if bit else 1 ^ C[v]

    for xs in range(8):
        e = 1
        for v in range(3):
            e = mul(e, f(v, (xs >> v) & 1))
        par, xs2, h = xs & 1, (xs >> 1) & 1, xs >> 2
        assert mul(mul(f(0, par), f(1, xs2)), f(2, h)) == e
        # and multiplying planes by a constant is linear: (a + b) E = a E + b E
        for y in (1, 0x53, 0xFF):
            assert mul(y, e) == mul(mul(y, mul(f(0, par), f(1, xs2))), f(2, h))


def test_acc9_reduce_formula():
    # csrc/zerocheck.cu acc9_reduce: a < 2^272 folded as L + H (1 + x + x^2 + x^7),
    # the bits of that above 127 folded once more; checked against long division
    import random
    M64 = (1 << 64) - 1
    POLY = (1 << 128) | 0x87

    def pmod(a):
        while a.bit_length() > 128:
            a ^= POLY << (a.bit_length() - 129)
        return a

    rng = random.Random(9)
    for _ in range(300):
        a = rng.getrandbits(255) << rng.randrange(16)  # a shifted 255-bit product
        l0, l1 = a & M64, (a >> 64) & M64
        h0, h1, h2 = (a >> 128) & M64, (a >> 192) & M64, a >> 256
        t0 = (h0 ^ (h0 << 1) ^ (h0 << 2) ^ (h0 << 7)) & M64
        t1 = (h1 ^ ((h1 << 1) | (h0 >> 63)) ^ ((h1 << 2) | (h0 >> 62)) ^ ((h1 << 7) | (h0 >> 57))) & M64
        t2 = (h2 ^ ((h2 << 1) | (h1 >> 63)) ^ ((h2 << 2) | (h1 >> 62)) ^ ((h2 << 7) | (h1 >> 57))) & M64
        lo = (l0 ^ t0 ^ t2 ^ (t2 << 1) ^ (t2 << 2) ^ (t2 << 7)) & M64
        hi = l1 ^ t1
        assert (hi << 64) | lo == pmod(a)


def test_lincheck_subset_sum_gray_walk():
    # csrc/lincheck.cu: thread (c, q) writes t8[8c + (i ^ (i >> 1))][q] for i < 8,
    # starting from the bits of 8c and adding weight ctz(i) at step i: every
    # entry v gets the XOR of the weights of its set bits, all 256 once
    import random
    rng = random.Random(4)
    w = [rng.getrandbits(128) for _ in range(8)]
    seen = {}
    for c in range(32):
        acc = 0
        for r in range(3, 8):
            if (c >> (r - 3)) & 1:
                acc ^= w[r]
        for i in range(8):
            if i:
                acc ^= w[0 if i & 1 else 1 if i & 2 else 2]
            seen[8 * c + (i ^ (i >> 1))] = acc
    assert sorted(seen) == list(range(256))
    for v, val in seen.items():
        want = 0
        for r in range(8):
            if (v >> r) & 1:
                want ^= w[r]
        assert val == want, v
