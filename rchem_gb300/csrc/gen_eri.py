"""Code generator for the Head-Gordon--Pople ERI class kernels.

For every angular-momentum class (la lb | lc ld) with la >= lb, lc >= ld and
l <= 2 per shell it writes straight-line code, templated on the real type R
(double for the FP64 form, float for the FP32 part of the mixed form):

* ``vrr_<cls>(...)``  -- Obara--Saika vertical recursion for one primitive
  quartet, from the scaled Boys values F[m] to [e0|f0]^(0) for every Cartesian
  e with la <= |e| <= la+lb and f with lc <= |f| <= lc+ld, added into the
  contraction accumulators ``acc``;
* ``hrr_<cls>(...)``  -- the horizontal recursion on the contracted
  accumulators, (a,b+1_i| = (a+1_i,b| + AB_i (a,b| on the bra and the same
  with CD on the ket, producing the (ab|cd) block in the reference's Cartesian
  order (src/shell.rs:1-12), each function scaled by its component
  normalisation factor (src/basis.rs:140-149 relative to the (l,0,0)
  component).

It also writes the per-class operation counts (FMA = 2 FLOP) that the
benchmark uses as the algorithmic FLOPs of a launch.  The algorithm follows
Head-Gordon & Pople (1988) and Obara & Saika (1986); the reference's own
implementation of the same recursions is libpyquante2/chgp.c:138-219,412-586.

Usage: python gen_eri.py OUTDIR
"""
from __future__ import annotations

import itertools
import os
import sys

LMAX = 2  # per shell (s, p, d)


def ijk_list(l):
    out = []
    for a in range(1, l + 2):
        for b in range(1, a + 1):
            out.append((l + 1 - a, a - b, b - 1))
    return out


def ncart(l):
    return (l + 1) * (l + 2) // 2


def comps_range(lo, hi):
    out = []
    for l in range(lo, hi + 1):
        out.extend(ijk_list(l))
    return out


def fact2(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def comp_norm(c):
    """N(alpha,l,m,n) / N(alpha,L,0,0)."""
    L = sum(c)
    return ((fact2(2 * L - 1)) / (fact2(2 * c[0] - 1) * fact2(2 * c[1] - 1) * fact2(2 * c[2] - 1))) ** 0.5


def sub(v, i, k=1):
    w = list(v)
    w[i] -= k
    return tuple(w)


def add(v, i, k=1):
    w = list(v)
    w[i] += k
    return tuple(w)


XYZ = "xyz"


def classes():
    pairs = [(a, b) for a in range(LMAX + 1) for b in range(a + 1)]  # ss ps pp ds dp dd
    pairs.sort(key=lambda ab: (ab[0] + ab[1], ab[0]))
    out = []
    for i, bra in enumerate(pairs):
        for ket in pairs[: i + 1]:
            out.append(bra + ket)
    return pairs, out


class Emitter:
    def __init__(self):
        self.lines = []
        self.names = {}
        self.nfma = 0  # fused multiply-adds
        self.nmul = 0  # plain multiplies / adds

    def emit(self, s):
        self.lines.append("    " + s)


def gen_vrr(la, lb, lc, ld, choose):
    """Returns (emitter, list of (target e, f) in accumulator order, L).

    The recurrence DAG is built first, then emitted as explicit FMA chains
    (``rchem_fma``: one DFMA each in FP64, a fused double-float operation in
    the emulated form).  A target integral that no other term reads is folded
    straight into its accumulator: acc = fma(X1, a, acc) ... instead of a
    product, the chain and a separate add, one instruction fewer per target and
    the same FLOPs."""
    E, F = la + lb, lc + ld
    L = E + F
    em = Emitter()
    memo = {}
    terms = {}   # node name -> list of terms
    order = []   # node names, children first
    uses = {}    # node name -> number of reads by other nodes
    coefs = set()

    def name(e, f, m):
        return "v_%d%d%d_%d%d%d_%d" % (e + f + (m,))

    def use(v):
        if not v.startswith("F["):
            uses[v] = uses.get(v, 0) + 1
        return v

    def coef(kind, n):
        if n == 1:
            return kind
        coefs.add((kind, n))
        return "%s_%d" % (kind, n)

    def node(e, f, m):
        key = (e, f, m)
        if key in memo:
            return memo[key]
        if sum(e) == 0 and sum(f) == 0:
            memo[key] = "F[%d]" % m
            return memo[key]
        # term kinds: ("mul", X, a) products, ("half", c, rho, a, b) = c*(a - rho*b)
        if sum(f) == 0:
            i = choose(e)
            e1 = sub(e, i)
            t = [("mul", "PA" + XYZ[i], node(e1, f, m)), ("mul", "WP" + XYZ[i], node(e1, f, m + 1))]
            nf, nm = 1, 1
            if e1[i] > 0:
                e2 = sub(e1, i)
                t.append(("half", coef("ohp", e1[i]), "rho_p", node(e2, f, m), node(e2, f, m + 1)))
                nf += 2
        else:
            i = choose(f)
            f1 = sub(f, i)
            t = [("mul", "QC" + XYZ[i], node(e, f1, m)), ("mul", "WQ" + XYZ[i], node(e, f1, m + 1))]
            nf, nm = 1, 1
            if f1[i] > 0:
                f2 = sub(f1, i)
                t.append(("half", coef("ohq", f1[i]), "rho_q", node(e, f2, m), node(e, f2, m + 1)))
                nf += 2
            if e[i] > 0:
                t.append(("mul", coef("ohpq", e[i]), node(sub(e, i), f1, m + 1)))
                nf += 1
        for term in t:
            for v in term[2:]:
                if term[0] == "mul" or v != term[2]:
                    use(v)
        nm_ = name(e, f, m)
        terms[nm_] = t
        order.append(nm_)
        em.nfma += nf
        em.nmul += nm
        memo[key] = nm_
        return nm_

    def chain(t, start):
        s_ = start
        for term in t:
            if term[0] == "mul":
                _, X, a = term
                s_ = "%s*%s" % (X, a) if s_ is None else "rchem_fma(%s, %s, %s)" % (X, a, s_)
            else:
                _, c, rho, a, b = term
                s_ = "rchem_fma(%s, rchem_fma(-%s, %s, %s), %s)" % (c, rho, b, a, s_)
        return s_

    targets = [(e, f) for e in comps_range(la, E) for f in comps_range(lc, F)]
    tnames = [node(e, f, 0) for (e, f) in targets]
    slot = {v: k for k, v in enumerate(tnames)}
    for kind, n in sorted(coefs):
        em.emit("const R %s_%d = R(%d)*%s;" % (kind, n, n, kind))
    folded = set()
    for v in order:
        if v in slot and uses.get(v, 0) == 0 and tnames.count(v) == 1:
            k = slot[v]
            em.emit("acc[%d] = %s;" % (k, chain(terms[v], "acc[%d]" % k)))
            folded.add(v)
        else:
            em.emit("const R %s = %s;" % (v, chain(terms[v], None)))
    for k, v in enumerate(tnames):
        if v not in folded:
            em.emit("acc[%d] += %s;" % (k, v))
        em.nmul += 1
    return em, targets, L


def gen_hrr(la, lb, lc, ld, targets, choose):
    """HRR on contracted accumulators -> out[] in (a,b,c,d) Cartesian order."""
    em = Emitter()
    E, F = la + lb, lc + ld
    eidx = {e: k for k, e in enumerate(comps_range(la, E))}
    fidx = {f: k for k, f in enumerate(comps_range(lc, F))}
    nf = len(fidx)
    # bra: (a,b|f) for every f in the ket accumulator range
    bra_memo = {}

    def bra(a, b, f):
        key = (a, b, f)
        if key in bra_memo:
            return bra_memo[key]
        if sum(b) == 0:
            s = "acc[%d]" % (eidx[a] * nf + fidx[f])
            bra_memo[key] = s
            return s
        i = choose(b)
        b1 = sub(b, i)
        x = bra(add(a, i), b1, f)
        y = bra(a, b1, f)
        nm = "hb_%d%d%d_%d%d%d_%d%d%d" % (a + b + f)
        em.emit("const R %s = rchem_fma(AB%s, %s, %s);" % (nm, XYZ[i], y, x))
        em.nfma += 1
        bra_memo[key] = nm
        return nm

    ket_memo = {}

    def ket(a, b, c, d):
        key = (a, b, c, d)
        if key in ket_memo:
            return ket_memo[key]
        if sum(d) == 0:
            s = bra(a, b, c)
            ket_memo[key] = s
            return s
        i = choose(d)
        d1 = sub(d, i)
        x = ket(a, b, add(c, i), d1)
        y = ket(a, b, c, d1)
        nm = "hk_%d%d%d_%d%d%d_%d%d%d_%d%d%d" % (a + b + c + d)
        em.emit("const R %s = rchem_fma(CD%s, %s, %s);" % (nm, XYZ[i], y, x))
        em.nfma += 1
        ket_memo[key] = nm
        return nm

    k = 0
    for a in ijk_list(la):
        for b in ijk_list(lb):
            for c in ijk_list(lc):
                for d in ijk_list(ld):
                    v = ket(a, b, c, d)
                    s = comp_norm(a) * comp_norm(b) * comp_norm(c) * comp_norm(d)
                    if abs(s - 1.0) < 1e-15:
                        em.emit("out[%d] = %s;" % (k, v))
                    else:
                        em.emit("out[%d] = R(%.17g)*%s;" % (k, s, v))
                        em.nmul += 1
                    k += 1
    return em


def choose_first(v):
    for i in range(3):
        if v[i] > 0:
            return i
    raise ValueError


def choose_last(v):
    for i in (2, 1, 0):
        if v[i] > 0:
            return i
    raise ValueError


def choose_max(v):
    best = max(v)
    for i in range(3):
        if v[i] == best:
            return i
    raise ValueError


CHOICES = {"first": choose_first, "last": choose_last, "max": choose_max}


def best_vrr(la, lb, lc, ld):
    best = None
    for nm, ch in CHOICES.items():
        em, targets, L = gen_vrr(la, lb, lc, ld, ch)
        cost = em.nfma + em.nmul
        if best is None or cost < best[0]:
            best = (cost, nm, em, targets, L)
    return best


def best_hrr(la, lb, lc, ld, targets):
    best = None
    for nm, ch in CHOICES.items():
        em = gen_hrr(la, lb, lc, ld, targets, ch)
        cost = em.nfma + em.nmul
        if best is None or cost < best[0]:
            best = (cost, nm, em)
    return best


# Boys-function cost model of boys.cuh (must stay in sync with it): a Horner
# chain of NTAY-1 FMAs per evaluated function; every F_m for L <= 1, else F_L
# and e^{-T} followed by the downward recursion (one FMA + one multiply per m);
# the prefactor multiplies (L+1 or 2); the grid index (one FMA + one add + one FMA).
NTAY64 = 5  # FP64 Boys table coefficients per row (boys.cuh)
NTAY32 = 4


def boys_ops(L, ntay=NTAY64):
    """(fma, other) FP64 operations of one Boys evaluation (boys_eval_u): x =
    grid - argument, one Horner chain per F_m (L <= 1) or for F_L and e^{-T}
    with the downward recursion (fma and a product per step, 2T once), and
    the products by the prefactor."""
    if L <= 1:
        return (ntay - 1) * (L + 1), 1 + (L + 1)
    return 2 * (ntay - 1) + L, 1 + 2 + 1 + L


def _split_args(s):
    """Top-level comma-separated arguments of s."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    out.append(cur.strip())
    return out


def _count_expr(e, seen):
    """(fma, other) of an emitted expression, each distinct subexpression once
    (the compiler evaluates a repeated one once)."""
    e = e.strip()
    while e.startswith("(") and e.endswith(")") and _split_args(e[1:-1]) == [e[1:-1].strip()]:
        e = e[1:-1].strip()
    if e.startswith("-") and "*" not in e and "rchem_fma" not in e:
        return 0, 0  # a negated operand: a sign modifier
    if e.startswith("rchem_fma("):
        f, o = (0, 0) if e in seen else (1, 0)
        seen.add(e)
        for a in _split_args(e[len("rchem_fma("):-1]):
            df, do = _count_expr(a, seen)
            f += df
            o += do
        return f, o
    depth = 0
    for i, ch in enumerate(e):
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == "*" and depth == 0:
            if e[:i].strip().startswith("R(") and e in seen:
                return 0, 0
            f, o = (0, 0) if e in seen else (0, 1)
            seen.add(e)
            for part in (e[:i], e[i + 1:]):
                df, do = _count_expr(part, seen)
                f += df
                o += do
            return f, o
    return 0, 0  # a leaf


def count_ops(lines):
    """(fma, other) FP64 operations of emitted statement lines (`lhs = expr;`)."""
    seen, f, o = set(), 0, 0
    for ln in lines:
        ln = ln.strip()
        if "=" not in ln or not ln.endswith(";"):
            continue
        rhs = ln.split("=", 1)[1].rstrip(";")
        if rhs.strip().startswith("R(") and "*" not in rhs:
            continue
        df, do = _count_expr(rhs, seen)
        f += df
        o += do
    return f, o


def setup_ops(la, lb, lc, ld):
    """(fma, other) FP64 operations of a primitive quartet before the Boys
    function, with 1/sqrt(p+q), pq/(p+q), q/(p+q), p/(p+q) from the exponent
    table: P - Q (3), |P - Q|^2 (a product and 2 FMA), T (1), the prefactor
    K_ab K_cd rs (2), W - P when the bra has angular momentum (3), W - Q when
    the ket has (3), 1/(2(p+q)) when both have (2).  (ss|ss) and (ps|ss) fold
    the prefactor and the W - P factor into their own products (their cases in
    eri_class_kernel)."""
    bra, ket = la + lb > 0, lc + ld > 0
    other = 3 + 1 + 1 + 2 + (3 if bra else 0) + (3 if ket else 0) + (2 if bra and ket else 0)
    return 2, other


# ---------------------------------------------------------------------------
# Warp-cooperative programs for the large classes.  Their straight-line VRR/HRR
# working sets (hundreds to thousands of intermediates) do not fit in one
# thread's registers; instead one warp evaluates one contracted quartet with
# the intermediates in shared memory, level by level of the recurrence DAG, the
# 32 lanes taking the independent terms of a level.  The DAG is the same one
# the straight-line code follows (same direction choices, same terms).
WC_MINL = 4  # classes with l_a+l_b+l_c+l_d >= WC_MINL get a program
WC_ONLY_MINL = 8  # ... and from here on have no one-lane-group-per-quartet kernel at all
# Total angular momenta whose one-lane-group kernel is a translation unit of
# its own, compiled with ptxas -O1: at -O3 the L = 6 kernels got 32 registers
# and ~19 KB of local memory per thread, at -O1 255 registers and ~3 KB, and
# ran twice as fast, and the L = 7 one ((dd|dp)) compiles in under a minute
# instead of minutes; the other kernels of these classes (warp-cooperative)
# stay at -O3, where they are faster.
SPLIT_L = (6, 7)


def _levels(depth, order, key):
    """Group node indices by depth; within a level sort by key (branch shape)."""
    by = {}
    for n in order:
        by.setdefault(depth[n], []).append(n)
    out, bounds = [], [0]
    for dlev in sorted(by):
        out.extend(sorted(by[dlev], key=key))
        bounds.append(len(out))
    return out, bounds


def _allocate(levels, last_read, fixed, nfixed):
    """Level-granular first-fit slot allocation.  ``levels``: node lists, level
    by level (a node reads only nodes of lower levels); ``last_read[n]``: the
    last level that reads n (absent: never read); ``fixed``: nodes that hold
    the slots [0, nfixed) from the start.  A slot is reused once every reader
    of its value has run, i.e. from the level after its last reader: within a
    level no term writes a slot another term of that level reads, so the lanes
    may take a level's terms in any order without synchronising.  Nodes in
    ``skip`` get no slot.  Returns ({node: slot}, slots used)."""
    import heapq

    slot = dict(fixed)
    free = []
    nslot = nfixed
    dying = {}
    for v, lv in last_read.items():
        dying.setdefault(lv, []).append(v)
    for k in range(nfixed):
        if k not in slot.values():
            heapq.heappush(free, k)
    for lev, nodes in enumerate(levels, start=1):
        for v in dying.get(lev - 1, []):
            if v in slot and slot[v] is not None:
                heapq.heappush(free, slot[v])
        for n in nodes:
            if n not in last_read:
                slot[n] = None
                continue
            if free:
                slot[n] = heapq.heappop(free)
            else:
                slot[n] = nslot
                nslot += 1
    return slot, nslot


def gen_prog(la, lb, lc, ld, choose_v, choose_h):
    """The warp-cooperative program of one class.  Per-warp shared memory is
    one array S of SCR values:
      VRR phase: S[0, NT) the [e0|f0] contraction accumulators, S[NT + m] the
        scaled Boys values F_m, the other VRR intermediates in S[NT + L + 1 ..);
      HRR phase: the accumulators are the inputs in place; intermediates and
        the outputs (ab|cd) take any dead slot, the outputs keeping theirs to
        the end (out[k] is the slot of output k).
    Slots are reused level by level (``_allocate``).  A VRR target is added
    into its accumulator by the term that computes it; it keeps a slot only
    if other terms read it.  Program words:
      VRR uint4: x = dest | a << 16, y = b | c << 16, z = d | g << 16,
                 w = dir | kind << 2 | n1 << 3 | n2 << 6 | (target + 1) << 9
                 (dest 0xffff: no store; target + 1 = 0: not a target);
      HRR uint2: x = dest | x << 16, y = y | dir << 16 | side << 24."""
    E, F = la + lb, lc + ld
    L = E + F
    idx, depth, recs, order = {}, {}, {}, []
    for m in range(L + 1):
        idx[((0, 0, 0), (0, 0, 0), m)] = m
        depth[m] = 0

    def node(e, f, m):
        key = (e, f, m)
        if key in idx:
            return idx[key]
        if sum(f) == 0:
            i = choose_v(e)
            e1 = sub(e, i)
            r = {"kind": 0, "dir": i, "a": node(e1, f, m), "b": node(e1, f, m + 1), "c": 0, "d": 0, "g": 0, "n1": 0, "n2": 0}
            if e1[i] > 0:
                e2 = sub(e1, i)
                r.update(c=node(e2, f, m), d=node(e2, f, m + 1), n1=e1[i])
        else:
            i = choose_v(f)
            f1 = sub(f, i)
            r = {"kind": 1, "dir": i, "a": node(e, f1, m), "b": node(e, f1, m + 1), "c": 0, "d": 0, "g": 0, "n1": 0, "n2": 0}
            if f1[i] > 0:
                f2 = sub(f1, i)
                r.update(c=node(e, f2, m), d=node(e, f2, m + 1), n1=f1[i])
            if e[i] > 0:
                r.update(g=node(sub(e, i), f1, m + 1), n2=e[i])
        k = L + 1 + len(order)
        kids = [r["a"], r["b"]] + ([r["c"], r["d"]] if r["n1"] else []) + ([r["g"]] if r["n2"] else [])
        depth[k] = 1 + max(depth[c] for c in kids)
        r["kids"] = kids
        recs[k] = r
        order.append(k)
        idx[key] = k
        return k

    targets = [(e, f) for e in comps_range(la, E) for f in comps_range(lc, F)]
    tgt = [node(e, f, 0) for (e, f) in targets]
    NT = len(targets)
    tgt_of = {}
    for t, n in enumerate(tgt):
        assert n > L, "a target is a Boys value: class too small for a program"
        tgt_of[n] = t
    vorder, vbounds = _levels(depth, order, lambda n: (recs[n]["kind"], recs[n]["n1"] > 0, recs[n]["n2"] > 0))
    vlevels = [vorder[vbounds[i]:vbounds[i + 1]] for i in range(len(vbounds) - 1)]
    vlast = {}
    for n in order:
        for c in recs[n]["kids"]:
            vlast[c] = max(vlast.get(c, 0), depth[n])
    for m in range(L + 1):
        vlast.setdefault(m, 0)
    vslot, vn = _allocate(vlevels, vlast, {m: m for m in range(L + 1)}, L + 1)
    vabs = lambda n: NT + vslot[n]  # noqa: E731

    eidx = {e: k for k, e in enumerate(comps_range(la, E))}
    fidx = {f: k for k, f in enumerate(comps_range(lc, F))}
    nf = len(fidx)
    hidx, hdepth, hrec, horder = {}, {}, {}, []
    for k in range(NT):
        hdepth[k] = 0

    def hnode(key, side, i, x, y):
        if key in hidx:
            return hidx[key]
        k = NT + len(horder)
        hdepth[k] = 1 + max(hdepth[x], hdepth[y])
        hrec[k] = {"side": side, "dir": i, "x": x, "y": y}
        horder.append(k)
        hidx[key] = k
        return k

    def bra(a, b, f):
        if sum(b) == 0:
            return eidx[a] * nf + fidx[f]
        key = ("b", a, b, f)
        if key in hidx:
            return hidx[key]
        i = choose_h(b)
        b1 = sub(b, i)
        return hnode(key, 0, i, bra(add(a, i), b1, f), bra(a, b1, f))

    def ket(a, b, c, d):
        if sum(d) == 0:
            return bra(a, b, c)
        key = ("k", a, b, c, d)
        if key in hidx:
            return hidx[key]
        i = choose_h(d)
        d1 = sub(d, i)
        return hnode(key, 1, i, ket(a, b, add(c, i), d1), ket(a, b, c, d1))

    outs = []
    for a in ijk_list(la):
        for b in ijk_list(lb):
            for c in ijk_list(lc):
                for d in ijk_list(ld):
                    outs.append((ket(a, b, c, d), comp_norm(a) * comp_norm(b) * comp_norm(c) * comp_norm(d)))
    NOUT = len(outs)
    horder2, hbounds = _levels(hdepth, horder, lambda n: hrec[n]["side"])
    hlevels = [horder2[hbounds[i]:hbounds[i + 1]] for i in range(len(hbounds) - 1)]
    assert len({n for n, _ in outs}) == NOUT, "a node is two outputs"
    hlast = {}
    for n in horder:
        for c in (hrec[n]["x"], hrec[n]["y"]):
            hlast[c] = max(hlast.get(c, 0), hdepth[n])
    for k in range(NT):
        hlast.setdefault(k, 0)
    for n, _ in outs:
        hlast[n] = len(hlevels) + 1  # outputs keep their slots to the end
    hslot, hn = _allocate(hlevels, hlast, {k: k for k in range(NT)}, NT)
    habs = lambda n: hslot[n]  # noqa: E731
    scr = max(NT + vn, hn)
    assert scr < 0xffff and NT < 2047
    # every level: distinct destinations, none of them read by the same level,
    # VRR destinations outside the accumulators
    for lv in vlevels:
        w = [vabs(n) for n in lv if vslot.get(n) is not None]
        rd = {vabs(c) for n in lv for c in recs[n]["kids"]}
        assert len(w) == len(set(w)) and not (set(w) & rd) and min(w + [NT]) >= NT
    for lv in hlevels:
        w = [habs(n) for n in lv]
        rd = {habs(c) for n in lv for c in (hrec[n]["x"], hrec[n]["y"])}
        assert len(w) == len(set(w)) and not (set(w) & rd) and max(w + [0]) < scr

    tag = "%d%d%d%d" % (la, lb, lc, ld)
    lines = ["// warp-cooperative program of class (%d%d|%d%d): %d VRR terms in %d levels, %d HRR terms in %d levels,"
             " %d shared values per warp" % (la, lb, lc, ld, len(order), len(vlevels), len(horder), len(hlevels), scr)]
    lines.append("static __device__ const uint4 rchem_vrr_%s[%d] = {" % (tag, len(vorder)))
    for n in vorder:
        r = recs[n]
        dest = vabs(n) if vslot.get(n) is not None else 0xffff
        g = vabs(r["g"]) if r["n2"] else 0
        c = vabs(r["c"]) if r["n1"] else 0
        d = vabs(r["d"]) if r["n1"] else 0
        t1 = tgt_of[n] + 1 if n in tgt_of else 0
        lines.append("  {%du, %du, %du, %du}," % (dest | (vabs(r["a"]) << 16), vabs(r["b"]) | (c << 16), d | (g << 16),
                                                  r["dir"] | (r["kind"] << 2) | (r["n1"] << 3) | (r["n2"] << 6) | (t1 << 9)))
    lines.append("};")
    lines.append("static __device__ const int rchem_vrrlv_%s[%d] = {%s};" % (tag, len(vbounds), ", ".join(map(str, vbounds))))
    lines.append("static __device__ const uint2 rchem_hrr_%s[%d] = {" % (tag, max(1, len(horder2))))
    for n in horder2:
        r = hrec[n]
        lines.append("  {%du, %du}," % (habs(n) | (habs(r["x"]) << 16), habs(r["y"]) | (r["dir"] << 16) | (r["side"] << 24)))
    if not horder2:
        lines.append("  {0u, 0u},")
    lines.append("};")
    lines.append("static __device__ const int rchem_hrrlv_%s[%d] = {%s};" % (tag, len(hbounds), ", ".join(map(str, hbounds))))
    lines.append("static __device__ const unsigned short rchem_out_%s[%d] = {%s};" % (tag, NOUT, ", ".join(str(habs(o[0])) for o in outs)))
    lines.append("static __device__ const double rchem_onorm_%s[%d] = {%s};" % (tag, NOUT, ", ".join("%.17g" % o[1] for o in outs)))
    lines.append("template <> struct EriProg<%d,%d,%d,%d> {" % (la, lb, lc, ld))
    lines.append("  static constexpr int NVL = %d, NHL = %d, NT = %d, NOUT = %d, SCR = %d;"
                 % (len(vlevels), len(hlevels), NT, NOUT, scr))
    for nm in ("vrr", "vrrlv", "hrr", "hrrlv", "out", "onorm"):
        ty = {"vrr": "uint4", "vrrlv": "int", "hrr": "uint2", "hrrlv": "int", "out": "unsigned short", "onorm": "double"}[nm]
        lines.append("  __device__ static __forceinline__ const %s *%s() { return rchem_%s_%s; }" % (ty, nm, nm, tag))
    lines.append("};")
    return lines


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    pairs, cls = classes()
    table = []
    for (la, lb, lc, ld) in cls:
        tag = "%d%d%d%d" % (la, lb, lc, ld)
        cost_v, chv, vem, targets, L = best_vrr(la, lb, lc, ld)
        cost_h, chh, hem = best_hrr(la, lb, lc, ld, targets)
        NE = len(comps_range(la, la + lb))
        NF = len(comps_range(lc, lc + ld))
        NA, NB, NC, ND = ncart(la), ncart(lb), ncart(lc), ncart(ld)
        # algorithmic FP64 operations of one primitive quartet, as the kernel
        # evaluates it: set-up, Boys function, the emitted VRR (each distinct
        # subexpression once); the two smallest classes by their own forms
        bf, bo = boys_ops(L)
        sf, so = setup_ops(la, lb, lc, ld)
        vf, vo = count_ops(vem.lines)
        if (la, lb, lc, ld) == (0, 0, 0, 0):  # pref F_0 into the accumulating FMA
            bo, vf, vo = bo - 1, 1, 0
        elif (la, lb, lc, ld) == (1, 0, 0, 0):  # PA_i (pref F_0) + PQ_i (-pref q/(p+q) F_1)
            so, bo, vf, vo = so - 3, bo + 1, 6, 0
        prim_flops = 2 * (vf + bf + sf) + (vo + bo + so)
        # per contracted quartet: HRR + scatter (6 FMA per integral)
        hf, ho = count_ops(hem.lines)
        contr_flops = 2 * hf + ho + 2 * 6 * NA * NB * NC * ND
        lines = []
        lines.append("// class (%d%d|%d%d): VRR %s-choice %d ops, HRR %s-choice %d ops" % (la, lb, lc, ld, chv, cost_v, chh, cost_h))
        lines.append("template <> struct EriClass<%d,%d,%d,%d> {" % (la, lb, lc, ld))
        lines.append("  static constexpr int L = %d, NE = %d, NF = %d, NA = %d, NB = %d, NC = %d, ND = %d;" % (L, NE, NF, NA, NB, NC, ND))
        lines.append("  static constexpr double PRIM_FLOPS = %d.0, CONTR_FLOPS = %d.0;" % (prim_flops, contr_flops))
        lines.append("  static constexpr bool WC = %s;  // a warp-cooperative program evaluates the J/K epilogue class"
                     % ("true" if L >= WC_MINL else "false"))
        lines.append("  static constexpr bool WC_ONLY = %s;  // every epilogue runs the warp-cooperative kernel"
                     % ("true" if L >= WC_ONLY_MINL else "false"))
        lines.append("  template <typename R> __host__ __device__ static __forceinline__ void vrr(R* __restrict__ acc, const R* __restrict__ F,")
        lines.append("      R PAx, R PAy, R PAz, R WPx, R WPy, R WPz, R QCx, R QCy, R QCz, R WQx, R WQy, R WQz,")
        lines.append("      R ohp, R ohq, R ohpq, R rho_p, R rho_q) {")
        lines.append("    (void)PAx; (void)PAy; (void)PAz; (void)WPx; (void)WPy; (void)WPz; (void)QCx; (void)QCy; (void)QCz;")
        lines.append("    (void)WQx; (void)WQy; (void)WQz; (void)ohp; (void)ohq; (void)ohpq; (void)rho_p; (void)rho_q;")
        lines.extend(vem.lines)
        lines.append("  }")
        lines.append("  template <typename R> __host__ __device__ static __forceinline__ void hrr(const R* __restrict__ acc, R* __restrict__ out,")
        lines.append("      R ABx, R ABy, R ABz, R CDx, R CDy, R CDz) {")
        lines.append("    (void)ABx; (void)ABy; (void)ABz; (void)CDx; (void)CDy; (void)CDz;")
        lines.extend(hem.lines)
        lines.append("  }")
        lines.append("};")
        if L >= WC_MINL:
            with open(os.path.join(outdir, "eri_prog_%s.inc" % tag), "w") as f:
                f.write("\n".join(gen_prog(la, lb, lc, ld, CHOICES[chv], CHOICES[chh])) + "\n")
        with open(os.path.join(outdir, "eri_class_%s.inc" % tag), "w") as f:
            f.write("\n".join(lines) + "\n")
        table.append((la, lb, lc, ld, prim_flops, contr_flops, NA * NB * NC * ND))
    # one translation unit per class (compiled in parallel); the classes of
    # total angular momentum in SPLIT_L put their one-lane-group kernel in a
    # second one, eri_<tag>_cls.cu, which build.py compiles with ptxas -O1
    for (la, lb, lc, ld) in cls:
        tag = "%d%d%d%d" % (la, lb, lc, ld)
        split = la + lb + lc + ld in SPLIT_L
        with open(os.path.join(outdir, "eri_%s.cu" % tag), "w") as f:
            f.write("// generated by gen_eri.py -- do not edit\n")
            f.write('#include "../eri_kernel.cuh"\n#include "eri_class_%s.inc"\n' % tag)
            if la + lb + lc + ld >= WC_MINL:
                f.write('#include "eri_prog_%s.inc"\n' % tag)
            if split:
                f.write("void rchem_launch_eri_cls_%s(const EriArgs &a, int prec, int epi, cudaStream_t s);"
                        "  // eri_%s_cls.cu\n" % (tag, tag))
            f.write("void rchem_launch_eri_%s(const EriArgs &a, int fp32, int epi, cudaStream_t s) {\n" % tag)
            if split:
                f.write("    launch_eri_class<%d, %d, %d, %d, true>(a, fp32, epi, s, rchem_launch_eri_cls_%s);\n}\n"
                        % (la, lb, lc, ld, tag))
            else:
                f.write("    launch_eri_class<%d, %d, %d, %d>(a, fp32, epi, s);\n}\n" % (la, lb, lc, ld))
            f.write("cudaError_t rchem_prepare_eri_%s() { return prepare_eri_class<%d, %d, %d, %d>(); }\n" % (tag, la, lb, lc, ld))
        if split:
            with open(os.path.join(outdir, "eri_%s_cls.cu" % tag), "w") as f:
                f.write("// generated by gen_eri.py -- do not edit\n")
                f.write('#include "../eri_kernel.cuh"\n#include "eri_class_%s.inc"\n' % tag)
                f.write("void rchem_launch_eri_cls_%s(const EriArgs &a, int prec, int epi, cudaStream_t s) {\n" % tag)
                f.write("    launch_eri_cls_only<%d, %d, %d, %d>(a, prec, epi, s);\n}\n" % (la, lb, lc, ld))
    with open(os.path.join(outdir, "eri_dispatch.h"), "w") as f:
        f.write("// generated by gen_eri.py -- do not edit\n#pragma once\n#include <cuda_runtime.h>\n")
        f.write('#include "../rchem_types.h"\n')
        for (la, lb, lc, ld) in cls:
            f.write("void rchem_launch_eri_%d%d%d%d(const EriArgs &a, int fp32, int epi, cudaStream_t s);\n" % (la, lb, lc, ld))
        for (la, lb, lc, ld) in cls:
            f.write("cudaError_t rchem_prepare_eri_%d%d%d%d();\n" % (la, lb, lc, ld))
        f.write("typedef cudaError_t (*rchem_eri_preparer)();\n")
        f.write("static const rchem_eri_preparer rchem_eri_prepare[%d] = {\n" % len(cls))
        for (la, lb, lc, ld) in cls:
            f.write("  rchem_prepare_eri_%d%d%d%d,\n" % (la, lb, lc, ld))
        f.write("};\n")
        f.write("typedef void (*rchem_eri_launcher)(const EriArgs &, int, int, cudaStream_t);\n")
        f.write("static const rchem_eri_launcher rchem_eri_launchers[%d] = {\n" % len(cls))
        for (la, lb, lc, ld) in cls:
            f.write("  rchem_launch_eri_%d%d%d%d,\n" % (la, lb, lc, ld))
        f.write("};\n")
    # index header
    with open(os.path.join(outdir, "eri_classes.h"), "w") as f:
        f.write("// generated by gen_eri.py -- do not edit\n#pragma once\n")
        f.write("#define RCHEM_NCLASS %d\n" % len(cls))
        f.write("static const int rchem_class_l[%d][4] = {\n" % len(cls))
        for t in table:
            f.write("  {%d,%d,%d,%d},\n" % t[:4])
        f.write("};\n")
        f.write("// 1: the J/K epilogue class runs the warp-cooperative program (one quartet per warp)\n")
        f.write("static const int rchem_class_wc[%d] = {%s};\n" % (
            len(cls), ", ".join("1" if sum(t[:4]) >= WC_MINL else "0" for t in table)))
        f.write("// 1: the class has only the warp-cooperative kernel (one quartet per warp in every plan)\n")
        f.write("static const int rchem_class_wc_only[%d] = {%s};\n" % (
            len(cls), ", ".join("1" if sum(t[:4]) >= WC_ONLY_MINL else "0" for t in table)))
        f.write("static const double rchem_class_flops[%d][2] = {\n" % len(cls))
        for t in table:
            f.write("  {%d.0, %d.0},\n" % t[4:6])
        f.write("};\n")
    return table


if __name__ == "__main__":
    tab = main(sys.argv[1] if len(sys.argv) > 1 else "_gen")
    for t in tab:
        print("(%d%d|%d%d) prim %6d flops  contr %7d flops  %4d ints" % t)
