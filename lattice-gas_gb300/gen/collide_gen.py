"""Collision-circuit generator: momentum classes -> LOP3-mapped CUDA.

The FHP rule is not hand-written.  As in the reference (src/collision.rs:62-69
enumerates the classes; src/gpu.rs:46-139 turns them into a Boolean circuit),
every cell state is grouped with the states of equal mass and momentum, and a
collision replaces a state by the member of its class that a random selector
picks:

  * class of size 2: fair bit s2; set -> class[0], clear -> class[1]
  * class of size 3: one-hot s3[0..2] -> class[k]; no bit set -> unchanged
  * class of size 5: one-hot s5[0..4] -> class[k]; no bit set -> unchanged
  * singleton classes: unchanged
(the known-answer specification at src/gpu.rs:799-817).  Without rest
particles the rule reads the six moving bits and passes bit 6 through.

What differs from the reference is how the rule becomes instructions.  The
reference emits a shared minterm prefix tree and ORs (685 two-input operators)
and leaves fusion to the shader compiler.  Here the rule is built as an
and-inverter graph (AIG) whose minterms come from the three opposite-direction
pairs (each pair is one of four states, so a six-bit minterm is a three-input
AND), and the AIG is covered with three-input lookup tables by a cut-based
technology mapper.  Each table is one `lop3.b32`, so the emitted instruction
count is known here, before anything runs.

The generator verifies its own output exhaustively (every state x every legal
selector, as the reference's KAT does) by simulating the mapped LUT network,
and emits `csrc/generated/collide.cuh`.

Usage:  python collide_gen.py [--out PATH] [--stats]
"""
from __future__ import annotations

import argparse
import os
import sys
from collections import defaultdict

CX2 = (2, 1, -1, -2, -1, 1)
CY2 = (0, 1, 1, 0, -1, -1)
REST = 6


# ---------------------------------------------------------------------------
# The rule (src/collision.rs:37-69)
# ---------------------------------------------------------------------------

def invariants(s: int):
    m = px = py = 0
    for d in range(6):
        if s >> d & 1:
            m += 1
            px += CX2[d]
            py += CY2[d]
    if s >> REST & 1:
        m += 1
    return (m, px, py)


def classes(rest: bool):
    """Classes ordered by (mass, px2, py2), states ascending within a class."""
    groups = defaultdict(list)
    for s in range(128 if rest else 64):
        groups[invariants(s)].append(s)
    return [groups[k] for k in sorted(groups)]


def rule(rest: bool, state: int, two: int, three: int, five: int) -> int:
    """The output of one lane (the reference's KAT statement, gpu.rs:803-813)."""
    hi = 0 if rest else state & 0x40
    s = state & (0x7F if rest else 0x3F)
    for g in classes(rest):
        if s in g:
            if len(g) == 2:
                out = g[0] if two else g[1]
            elif len(g) == 3:
                out = g[three] if three < 3 else s
            elif len(g) == 5:
                out = g[five] if five < 5 else s
            else:
                out = s
            return out | hi
    raise AssertionError


# ---------------------------------------------------------------------------
# And-inverter graph with structural hashing.  A literal is 2*node + neg.
# Node 0 is constant false, so literal 0 = false and 1 = true.
# ---------------------------------------------------------------------------

class AIG:
    def __init__(self):
        self.fanins = [None]          # node 0: constant
        self.names = ["0"]
        self.inputs = []              # node ids of primary inputs
        self.table = {}

    def input(self, name):
        self.fanins.append(None)
        self.names.append(name)
        nid = len(self.fanins) - 1
        self.inputs.append(nid)
        return 2 * nid

    def AND(self, a, b):
        if a > b:
            a, b = b, a
        if a == 0:
            return 0
        if a == 1:
            return b
        if a == b:
            return a
        if a ^ 1 == b:
            return 0
        key = (a, b)
        if key in self.table:
            return self.table[key]
        self.fanins.append(key)
        self.names.append(None)
        lit = 2 * (len(self.fanins) - 1)
        self.table[key] = lit
        return lit

    @staticmethod
    def NOT(a):
        return a ^ 1

    def OR(self, a, b):
        return self.AND(a ^ 1, b ^ 1) ^ 1

    def AND_n(self, lits):
        lits = list(lits)
        if not lits:
            return 1
        while len(lits) > 1:
            nxt = [self.AND(lits[i], lits[i + 1]) for i in range(0, len(lits) - 1, 2)]
            if len(lits) % 2:
                nxt.append(lits[-1])
            lits = nxt
        return lits[0]

    def OR_n(self, lits):
        return self.AND_n([x ^ 1 for x in lits]) ^ 1

    def MUX(self, s, a, b):
        """s ? a : b"""
        return self.OR(self.AND(s, a), self.AND(s ^ 1, b))


def build_rule_aig(rest: bool):
    g = AIG()
    n = [g.input("n%d" % d) for d in range(7)]
    s2 = g.input("s2")
    s3 = [g.input("s3_%d" % k) for k in range(3)]
    s5 = [g.input("s5_%d" % k) for k in range(5)]

    # Opposite-direction pairs (d, d+3): four exclusive states each.
    pair = []
    for k in range(3):
        lo, hi = n[k], n[k + 3]
        pair.append({(0, 0): g.AND(lo ^ 1, hi ^ 1), (1, 0): g.AND(lo, hi ^ 1),
                     (0, 1): g.AND(lo ^ 1, hi), (1, 1): g.AND(lo, hi)})

    def minterm6(s):
        ps = [pair[k][(s >> k & 1, s >> (k + 3) & 1)] for k in range(3)]
        return g.AND(ps[0], g.AND(ps[1], ps[2]))

    def member_set(states):
        """Indicator of a set of 7-bit (or 6-bit) states."""
        if not rest:
            return g.OR_n([minterm6(s) for s in states])
        r0 = [s for s in states if not s >> REST & 1]
        r1 = [s & 0x3F for s in states if s >> REST & 1]
        t0 = g.OR_n([minterm6(s) for s in r0]) if r0 else 0
        t1 = g.OR_n([minterm6(s) for s in r1]) if r1 else 0
        return g.OR(g.AND(n[REST] ^ 1, t0), g.AND(n[REST], t1))

    cls = [c for c in classes(rest) if len(c) > 1]
    for c in cls:
        assert len(c) in (2, 3, 5), "no selector for a class of %d states" % len(c)
    ind = {tuple(c): member_set(c) for c in cls}

    nbits = 7 if rest else 6
    any3 = g.OR_n(s3)
    any5 = g.OR_n(s5)
    by_size = {2: [], 3: [], 5: []}
    for c in cls:
        by_size[len(c)].append(c)

    acted = []
    if by_size[2]:
        acted.append(g.OR_n([ind[tuple(c)] for c in by_size[2]]))
    if by_size[3]:
        acted.append(g.AND(g.OR_n([ind[tuple(c)] for c in by_size[3]]), any3))
    if by_size[5]:
        acted.append(g.AND(g.OR_n([ind[tuple(c)] for c in by_size[5]]), any5))
    keep = g.OR_n(acted) ^ 1

    outs = []
    for d in range(7):
        if d >= nbits:
            outs.append(n[d])
            continue
        terms = [g.AND(n[d], keep)]
        # size 2: s2 ? A : B
        A = g.OR_n([ind[tuple(c)] for c in by_size[2] if c[0] >> d & 1])
        B = g.OR_n([ind[tuple(c)] for c in by_size[2] if c[1] >> d & 1])
        terms.append(g.MUX(s2, A, B))
        for size, sel in ((3, s3), (5, s5)):
            for k in range(size):
                X = g.OR_n([ind[tuple(c)] for c in by_size[size] if c[k] >> d & 1])
                terms.append(g.AND(sel[k], X))
        outs.append(g.OR_n(terms))
    return g, outs


def build_rule_aig_folded(order=(2, 0, 1), reverse_terms=True):
    """FHP-III rule through its particle-hole symmetry.

    Complementing all seven bits maps class (m, px2, py2) onto (7 - m, -px2,
    -py2) and reverses the ascending member order, so
    class'[k] = ~class[size - 1 - k].  With z = [mass >= 4] (bit 2 of the
    population count), the circuit evaluates only the fourteen classes of
    mass 2 and 3 on m = n ^ z, with the selectors order-reversed where z is
    set (s2 -> ~s2, s3[k] -> s3[2-k], s5[k] -> s5[4-k]), and complements the
    picked member back.  Singleton classes map onto singleton classes, so a
    lane with nothing to do keeps its state whatever z is.
    """
    g = AIG()
    n = [g.input("n%d" % d) for d in range(7)]
    s2 = g.input("s2")
    s3 = [g.input("s3_%d" % k) for k in range(3)]
    s5 = [g.input("s5_%d" % k) for k in range(5)]

    def XOR(a, b):
        return g.OR(g.AND(a, b ^ 1), g.AND(a ^ 1, b))

    def MAJ(a, b, c):
        return g.OR(g.AND(a, b), g.AND(c, g.OR(a, b)))

    # bit 2 of popcount(n0..n6) by full adders
    s_a = XOR(XOR(n[0], n[1]), n[2])
    c_a = MAJ(n[0], n[1], n[2])
    s_b = XOR(XOR(n[3], n[4]), n[5])
    c_b = MAJ(n[3], n[4], n[5])
    c_c = MAJ(s_a, s_b, n[6])
    z = MAJ(c_a, c_b, c_c)

    m = [XOR(n[d], z) for d in range(7)]
    t2 = XOR(s2, z)
    t3 = [g.MUX(z, s3[2 - k], s3[k]) for k in range(3)]
    t5 = [g.MUX(z, s5[4 - k], s5[k]) for k in range(5)]

    pair = []
    for k in range(3):
        lo, hi = m[k], m[k + 3]
        pair.append({(0, 0): g.AND(lo ^ 1, hi ^ 1), (1, 0): g.AND(lo, hi ^ 1),
                     (0, 1): g.AND(lo ^ 1, hi), (1, 1): g.AND(lo, hi)})

    def minterm6(s):
        ps = [pair[k][(s >> k & 1, s >> (k + 3) & 1)] for k in range(3)]
        a, b, c = (ps[i] for i in order)
        return g.AND(a, g.AND(b, c))

    def member_set(states):
        r0 = [s for s in states if not s >> REST & 1]
        r1 = [s & 0x3F for s in states if s >> REST & 1]
        a = g.OR_n([minterm6(s) for s in r0]) if r0 else 0
        b = g.OR_n([minterm6(s) for s in r1]) if r1 else 0
        return g.OR(g.AND(m[REST] ^ 1, a), g.AND(m[REST], b))

    lower = [c for c in classes(True) if len(c) > 1 and invariants(c[0])[0] <= 3]
    assert len(lower) == 14
    ind = {tuple(c): member_set(c) for c in lower}
    by_size = {2: [], 3: [], 5: []}
    for c in lower:
        by_size[len(c)].append(c)
    any3 = g.OR_n(s3)
    any5 = g.OR_n(s5)
    acted = [g.OR_n([ind[tuple(c)] for c in by_size[2]]),
             g.AND(g.OR_n([ind[tuple(c)] for c in by_size[3]]), any3),
             g.AND(g.OR_n([ind[tuple(c)] for c in by_size[5]]), any5)]
    keep = g.OR_n(acted) ^ 1
    outs = []
    for d in range(7):
        A = g.OR_n([ind[tuple(c)] for c in by_size[2] if c[0] >> d & 1])
        B = g.OR_n([ind[tuple(c)] for c in by_size[2] if c[1] >> d & 1])
        terms = [g.MUX(t2, A, B)]
        for size, sel in ((3, t3), (5, t5)):
            for k in range(size):
                X = g.OR_n([ind[tuple(c)] for c in by_size[size] if c[k] >> d & 1])
                terms.append(g.AND(sel[k], X))
        if reverse_terms:
            terms = terms[::-1]
        target = XOR(g.OR_n(terms), z)
        outs.append(g.MUX(keep, n[d], target))
    return g, outs


def build_selector_aig():
    """One-hot selectors from the hash chain (src/gpu.rs:157-180) in nested form.

    The reference accumulates s3[j] |= open & f_j(a, b) round by round with
    open &= a & b (and s5 likewise with open5 &= c & (a | b)).  The rounds are
    nested, so the same selectors are
        s3[j] = f_j(r0) | g(r0) & (f_j(r1) | g(r1) & f_j(r2))
    with g the continue condition of a round; that form maps onto fewer
    three-input tables.  Inputs r1..r18 are the 2nd..19th hashes of the chain.
    """
    g = AIG()
    r = [None] + [g.input("r%d" % i) for i in range(1, 19)]
    f3 = [lambda a, b: g.AND(a ^ 1, b ^ 1), lambda a, b: g.AND(a, b ^ 1),
          lambda a, b: g.AND(a ^ 1, b)]
    c3 = lambda a, b: g.AND(a, b)
    rounds3 = [(r[1], r[2]), (r[3], r[4]), (r[5], r[6])]
    outs = []
    for j in range(3):
        acc = f3[j](*rounds3[2])
        for a, b in (rounds3[1], rounds3[0]):
            acc = g.OR(f3[j](a, b), g.AND(c3(a, b), acc))
        outs.append(acc)
    f5 = [lambda a, b, c: g.AND_n([a ^ 1, b ^ 1, c ^ 1]), lambda a, b, c: g.AND_n([a, b ^ 1, c ^ 1]),
          lambda a, b, c: g.AND_n([a ^ 1, b, c ^ 1]), lambda a, b, c: g.AND_n([a, b, c ^ 1]),
          lambda a, b, c: g.AND_n([a ^ 1, b ^ 1, c])]
    c5 = lambda a, b, c: g.AND(c, g.OR(a, b))
    rounds5 = [(r[7], r[8], r[9]), (r[10], r[11], r[12]), (r[13], r[14], r[15]),
               (r[16], r[17], r[18])]
    for j in range(5):
        acc = f5[j](*rounds5[3])
        for rd in (rounds5[2], rounds5[1], rounds5[0]):
            acc = g.OR(f5[j](*rd), g.AND(c5(*rd), acc))
        outs.append(acc)
    return g, outs


def selector_reference(rs):
    """The reference's accumulate-with-mask form, for verification."""
    M = (1 << 64) - 1
    s3 = [0, 0, 0]
    open_ = M
    for k in range(3):
        a, b = rs[1 + 2 * k], rs[2 + 2 * k]
        s3[0] |= open_ & ~a & ~b & M
        s3[1] |= open_ & a & ~b & M
        s3[2] |= open_ & ~a & b & M
        open_ &= a & b
    s5 = [0] * 5
    open5 = M
    for k in range(4):
        a, b, c = rs[7 + 3 * k], rs[8 + 3 * k], rs[9 + 3 * k]
        s5[0] |= open5 & ~a & ~b & ~c & M
        s5[1] |= open5 & a & ~b & ~c & M
        s5[2] |= open5 & ~a & b & ~c & M
        s5[3] |= open5 & a & b & ~c & M
        s5[4] |= open5 & ~a & ~b & c & M
        open5 &= c & (a | b)
    return s3 + s5


def verify_selectors(g, luts, outs):
    """Exhaustive per lane: all 2^12 bit patterns of the s5 rounds, each lane
    also carrying one of the 2^6 patterns of the s3 rounds."""
    for base in range(0, 4096, 64):
        rs = [None] + [0] * 18
        for lane in range(64):
            i = base + lane
            for b in range(6):
                if (i % 64) >> b & 1:
                    rs[1 + b] |= 1 << lane
            for b in range(12):
                if i >> b & 1:
                    rs[7 + b] |= 1 << lane
        if eval_luts(g, luts, outs, rs[1:]) != selector_reference(rs):
            return False
    return True


# ---------------------------------------------------------------------------
# Cut-based mapping onto three-input LUTs (one lop3 each).
# ---------------------------------------------------------------------------

def map_lut3(g: AIG, outs):
    nn = len(g.fanins)
    is_input = [False] * nn
    for i in g.inputs:
        is_input[i] = True
    is_input[0] = True
    # reachable nodes in topological order (node ids are already topological)
    need = [False] * nn
    stack = [o >> 1 for o in outs]
    while stack:
        v = stack.pop()
        if need[v]:
            continue
        need[v] = True
        if g.fanins[v] is not None:
            stack.append(g.fanins[v][0] >> 1)
            stack.append(g.fanins[v][1] >> 1)
    order = [v for v in range(nn) if need[v]]
    fanout = [0] * nn
    for v in order:
        if g.fanins[v] is not None:
            fanout[g.fanins[v][0] >> 1] += 1
            fanout[g.fanins[v][1] >> 1] += 1
    for o in outs:
        fanout[o >> 1] += 1

    cuts = {}
    for v in order:
        if is_input[v]:
            cuts[v] = [frozenset([v])] if v != 0 else [frozenset()]
            continue
        a, b = g.fanins[v]
        cs = set()
        for ca in cuts[a >> 1]:
            for cb in cuts[b >> 1]:
                u = ca | cb
                if len(u) <= 3:
                    cs.add(u)
        # drop dominated cuts
        cl = sorted(cs, key=len)
        kept = []
        for c in cl:
            if not any(k <= c for k in kept):
                kept.append(c)
        kept.append(frozenset([v]))
        cuts[v] = kept

    def best_cover(ref_weight):
        """Area-flow selection; returns chosen cut per node."""
        af = {}
        choice = {}
        for v in order:
            if is_input[v]:
                af[v] = 0.0
                continue
            best = None
            for c in cuts[v]:
                if c == frozenset([v]):
                    continue
                cost = 1.0 + sum(af[l] / max(ref_weight(l), 1) for l in c)
                if best is None or cost < best[0] - 1e-9 or (abs(cost - best[0]) < 1e-9 and len(c) < len(best[1])):
                    best = (cost, c)
            af[v] = best[0]
            choice[v] = best[1]
        return choice

    def cover_from(choice):
        used = set()
        stack = [o >> 1 for o in outs]
        while stack:
            v = stack.pop()
            if is_input[v] or v in used:
                continue
            used.add(v)
            stack.extend(choice[v])
        return used

    choice = best_cover(lambda l: fanout[l])
    used = cover_from(choice)
    # area recovery: re-run with reference counts from the current cover
    for _ in range(4):
        refs = defaultdict(int)
        for v in used:
            for l in choice[v]:
                refs[l] += 1
        for o in outs:
            refs[o >> 1] += 1
        choice2 = best_cover(lambda l: refs.get(l, fanout[l]) or fanout[l])
        used2 = cover_from(choice2)
        if len(used2) < len(used):
            choice, used = choice2, used2
        else:
            break

    # truth tables: leaves get 0xF0, 0xCC, 0xAA (lop3's a, b, c)
    luts = []
    for v in sorted(used):
        leaves = sorted(choice[v])
        tt_leaf = dict(zip(leaves, (0xF0, 0xCC, 0xAA)))
        memo = {}

        def tt(u):
            if u in tt_leaf:
                return tt_leaf[u]
            if u == 0:
                return 0
            if u in memo:
                return memo[u]
            a, b = g.fanins[u]
            ta = tt(a >> 1) ^ (0xFF if a & 1 else 0)
            tb = tt(b >> 1) ^ (0xFF if b & 1 else 0)
            memo[u] = ta & tb
            return memo[u]

        luts.append((v, leaves, tt(v)))
    return luts


# ---------------------------------------------------------------------------
# Simulation and verification
# ---------------------------------------------------------------------------

def eval_luts(g, luts, outs, input_words):
    """Evaluate on 64-bit words (one test vector per lane)."""
    M = (1 << 64) - 1
    val = {0: 0}
    for nid, w in zip(g.inputs, input_words):
        val[nid] = w
    for v, leaves, table in luts:
        xs = [val[l] for l in leaves] + [0] * (3 - len(leaves))
        a, b, c = xs
        r = 0
        for i in range(8):
            if table >> i & 1:
                ta = a if i & 4 else ~a & M
                tb = b if i & 2 else ~b & M
                tc = c if i & 1 else ~c & M
                r |= ta & tb & tc
        val[v] = r
    res = []
    for o in outs:
        x = val[o >> 1]
        res.append(x ^ M if o & 1 else x)
    return res


def verify(rest, g, luts, outs):
    """Every state x every legal selector (the reference KAT's domain)."""
    n_states = 128 if rest else 64
    combos = [(s, two, three, five) for s in range(n_states) for two in (0, 1)
              for three in range(4) for five in range(6)]
    # also the no-rest rule must pass the rest bit through for states >= 64
    if not rest:
        combos += [(s | 0x40, two, three, five) for s in range(64) for two in (0, 1)
                   for three in range(4) for five in range(6)]
    bad = 0
    for base in range(0, len(combos), 64):
        chunk = combos[base:base + 64]
        words = [0] * 16
        for lane, (s, two, three, five) in enumerate(chunk):
            bit = 1 << lane
            for d in range(7):
                if s >> d & 1:
                    words[d] |= bit
            if two:
                words[7] |= bit
            if three < 3:
                words[8 + three] |= bit
            if five < 5:
                words[11 + five] |= bit
        res = eval_luts(g, luts, outs, words)
        for lane, (s, two, three, five) in enumerate(chunk):
            got = sum(((res[d] >> lane) & 1) << d for d in range(7))
            want = rule(rest, s, two, three, five)
            if got != want:
                bad += 1
    return len(combos), bad


# ---------------------------------------------------------------------------
# Emission
# ---------------------------------------------------------------------------

def emit(rest, g, luts, outs, fname):
    names = {}
    for nid in g.inputs:
        names[nid] = g.names[nid]
    lines = []
    lines.append("// %s: %d lop3 per 32-cell word (rest particles: %s)"
                 % (fname, len(luts), "yes" if rest else "no"))
    lines.append("LGX_HD_INLINE void %s(const uint32_t n[7], uint32_t s2, const uint32_t s3[3],"
                 % fname)
    lines.append("                      const uint32_t s5[5], uint32_t o[7]) {")
    used = set()
    for _, leaves, _ in luts:
        used.update(leaves)
    used.update(o >> 1 for o in outs)
    src_of = {"s2": None}
    for d in range(7):
        src_of["n%d" % d] = "n[%d]" % d
    for k in range(3):
        src_of["s3_%d" % k] = "s3[%d]" % k
    for k in range(5):
        src_of["s5_%d" % k] = "s5[%d]" % k
    for nid in g.inputs:
        nm = g.names[nid]
        if nid in used and src_of[nm] is not None:
            lines.append("  const uint32_t %s = %s;" % (nm, src_of[nm]))
    if not any(g.names[nid] == "s2" and nid in used for nid in g.inputs):
        lines.append("  (void)s2;")
    if not any(g.names[nid].startswith("s3") and nid in used for nid in g.inputs):
        lines.append("  (void)s3;")
    if not any(g.names[nid].startswith("s5") and nid in used for nid in g.inputs):
        lines.append("  (void)s5;")
    for v, leaves, table in luts:
        names[v] = "t%d" % v
        args = [names[l] for l in leaves] + ["0u"] * (3 - len(leaves))
        lines.append("  const uint32_t t%d = LGX_LOP3(%s, %s, %s, 0x%02x);"
                     % (v, args[0], args[1], args[2], table))
    for d, o in enumerate(outs):
        v = o >> 1
        src = names[v] if v != 0 else "0u"
        lines.append("  o[%d] = %s%s;" % (d, "~" if o & 1 else "", src))
    lines.append("}")
    return "\n".join(lines)


def emit_selectors(g, luts, outs):
    names = {nid: g.names[nid] for nid in g.inputs}
    lines = ["// lgx_selectors: %d lop3; r[0..17] are hashes 2..19 of the chain" % len(luts),
             "LGX_HD_INLINE void lgx_selectors(const uint32_t r[18], uint32_t s3[3], uint32_t s5[5]) {"]
    used = set()
    for _, leaves, _ in luts:
        used.update(leaves)
    for nid in g.inputs:
        if nid in used:
            lines.append("  const uint32_t %s = r[%d];" % (names[nid], int(names[nid][1:]) - 1))
    for v, leaves, table in luts:
        names[v] = "t%d" % v
        args = [names[l] for l in leaves] + ["0u"] * (3 - len(leaves))
        lines.append("  const uint32_t t%d = LGX_LOP3(%s, %s, %s, 0x%02x);"
                     % (v, args[0], args[1], args[2], table))
    dst = ["s3[0]", "s3[1]", "s3[2]", "s5[0]", "s5[1]", "s5[2]", "s5[3]", "s5[4]"]
    for d, o in zip(dst, outs):
        lines.append("  %s = %s%s;" % (d, "~" if o & 1 else "", names[o >> 1]))
    lines.append("}")
    return "\n".join(lines)


HEADER = """// Generated by lattice-gas_gb300/gen/collide_gen.py -- do not edit.
//
// The FHP collision rule as three-input lookup tables, one lop3.b32 each.
// Inputs: seven planes n[0..6] (six directions, then rest), the fair bit s2,
// one-hot selectors s3[0..2] and s5[0..4].  Output: seven planes o[0..6].
// Semantics (class pick by selector) follow the reference's known-answer
// specification, src/gpu.rs:799-817; classes come from src/collision.rs:62-69.
#pragma once
#include <stdint.h>

#ifndef LGX_HD_INLINE
#if defined(__CUDACC__)
#define LGX_HD_INLINE __host__ __device__ __forceinline__
#else
#define LGX_HD_INLINE static inline
#endif
#endif

#define LGX_LOP3(a, b, c, lut) lgx_lop3_host((a), (b), (c), (lut))

// Host evaluation of a three-input table: bit i of lut is f(a_i, b_i, c_i)
// with i = 4a + 2b + c (the lop3 convention: a = 0xF0, b = 0xCC, c = 0xAA).
static inline uint32_t lgx_lop3_host(uint32_t a, uint32_t b, uint32_t c, uint32_t lut) {
  uint32_t r = 0;
  for (int i = 0; i < 8; ++i) {
    if ((lut >> i) & 1u) {
      uint32_t ta = (i & 4) ? a : ~a, tb = (i & 2) ? b : ~b, tc = (i & 1) ? c : ~c;
      r |= ta & tb & tc;
    }
  }
  return r;
}
"""


def lop3_device_helpers(tables):
    out = ["#if defined(__CUDA_ARCH__)"]
    for t in sorted(tables):
        out.append("__device__ __forceinline__ uint32_t lgx_lop3_0x%02x(uint32_t a, uint32_t b, "
                   "uint32_t c) {" % t)
        out.append("  uint32_t r;")
        out.append('  asm("lop3.b32 %%0, %%1, %%2, %%3, 0x%02x;" : "=r"(r) : "r"(a), "r"(b), '
                   '"r"(c));' % t)
        out.append("  return r;")
        out.append("}")
    out.append("#endif")
    return "\n".join(out)


def generate(stats=False):
    parts = []
    tables = set()
    bodies = []
    report = {}
    for rest, fname in ((True, "lgx_collide_rest"), (False, "lgx_collide_norest")):
        # Without rest particles mass 3 is its own complement, so the folded
        # form would not halve anything; that rule is built directly.
        g, outs = build_rule_aig_folded() if rest else build_rule_aig(rest)
        luts = map_lut3(g, outs)
        total, bad = verify(rest, g, luts, outs)
        if bad:
            raise SystemExit("generated rule disagrees with the enumeration on %d of %d cases"
                             % (bad, total))
        ands = sum(1 for f in g.fanins if f is not None)
        report[fname] = dict(aig_ands=ands, lop3=len(luts), checked=total)
        for _, _, t in luts:
            tables.add(t)
        bodies.append(emit(rest, g, luts, outs, fname))
    gs, souts = build_selector_aig()
    sluts = map_lut3(gs, souts)
    if not verify_selectors(gs, sluts, souts):
        raise SystemExit("generated selectors disagree with the reference's rejection sampling")
    report["lgx_selectors"] = dict(aig_ands=sum(1 for f in gs.fanins if f is not None),
                                   lop3=len(sluts), checked=64 * 64)
    for _, _, t in sluts:
        tables.add(t)
    bodies.append(emit_selectors(gs, sluts, souts))
    parts.append(HEADER)
    parts.append(lop3_device_helpers(tables))
    parts.append("#if defined(__CUDA_ARCH__)")
    parts.append("#undef LGX_LOP3")
    parts.append("#define LGX_LOP3(a, b, c, lut) lgx_lop3_##lut(a, b, c)")
    parts.append("#endif")
    for b in bodies:
        parts.append(b)
    parts.append("// stats: " + "; ".join("%s %s" % (k, v) for k, v in report.items()))
    src = "\n\n".join(parts) + "\n"
    if stats:
        for k, v in report.items():
            print(k, v, file=sys.stderr)
    return src, report


def main():
    ap = argparse.ArgumentParser()
    here = os.path.dirname(os.path.abspath(__file__))
    ap.add_argument("--out", default=os.path.join(here, "..", "csrc", "generated", "collide.cuh"))
    ap.add_argument("--stats", action="store_true")
    args = ap.parse_args()
    src, _ = generate(stats=args.stats)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    old = open(args.out).read() if os.path.exists(args.out) else None
    if old != src:
        with open(args.out, "w") as f:
            f.write(src)


if __name__ == "__main__":
    main()
