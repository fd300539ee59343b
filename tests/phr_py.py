"""A second, pure-Python restatement of PHR (pkg/pt/phr.go:47-459), used only
to cross-check the C oracle on small inputs.  It rebuilds the auxiliary tree
from the oracle's pre-order export, runs the refinement with the same FIFO
initial cut, and exports the result in the same pre-order format.
"""
import sys
from collections import deque

import numpy as np

MAX_CUT_SIZE = 2500  # phr.go:11


class Aux:
    __slots__ = ("leaf", "box", "kids", "prims", "size", "bc")


class Out:
    __slots__ = ("leaf", "box", "kids", "prims")

    def __init__(self, leaf, box, kids=None, prims=None):
        self.leaf, self.box, self.kids, self.prims = leaf, box, kids or [], prims or []


def surface(b):  # bounding.go:45-47
    w, h, d = b[3] - b[0], b[4] - b[1], b[5] - b[2]
    return 2 * w * h + 2 * w * d + 2 * h * d


def add(a, b):  # MinVec / MaxVec
    lo = [a[k] if not (a[k] > b[k]) else b[k] for k in range(3)]
    hi = [a[3 + k] if not (a[3 + k] < b[3 + k]) else b[3 + k] for k in range(3)]
    return tuple(lo + hi)


def parse(kind, count, box, prims):
    sys.setrecursionlimit(100000)
    pos = [0, 0]

    def rec():
        i = pos[0]
        pos[0] += 1
        n = Aux()
        n.leaf = bool(kind[i])
        n.box = tuple(float(x) for x in box[i])
        n.bc = tuple((n.box[k] + n.box[3 + k]) * 0.5 for k in range(3))
        if n.leaf:
            c = int(count[i])
            n.prims = [int(p) for p in prims[pos[1]:pos[1] + c]]
            pos[1] += c
            n.kids = []
            n.size = 1
        else:
            n.kids = [rec() for _ in range(int(count[i]))]
            n.prims = []
            n.size = 1 + sum(k.size for k in n.kids)
        return n

    return rec()


def collect(n, acc):
    if isinstance(n, Out):
        acc.extend(n.prims)
    elif n.leaf:
        acc.extend(n.prims)
    else:
        for k in n.kids:
            collect(k, acc)


def phr(root, alpha, delta, bf, stats=None):
    """stats, if a dict, receives build_cost: BuildWithCost's count (phr.go:154-255), the
    initial cut's size plus the size of every cut handed to Split."""
    S = surface(root.box)
    cost = [0]

    def thr(depth):  # DefaultThreshold
        return S / (2.0 ** (alpha * float(depth) + delta))

    def make_leaf(box, nodes):
        acc = []
        for n in nodes:
            collect(n, acc)
        return Out(True, box, prims=acc)

    def refined(cut):
        nodes, box, depth = cut
        t = thr(depth)
        r = []
        for n in nodes:
            if isinstance(n, Out) or n.leaf or surface(n.box) < t:
                r.append(n)
            else:
                r.extend(n.kids)
        if len(r) == 1:
            r = [make_leaf(box, r)]
        return (r, box, depth + 1)

    def min_cost(s, box, depth):
        n = len(s)
        sa_right = s[n - 1].box
        rc = [0.0] * n
        rb = [None] * n
        count = 0
        for i in range(n - 1, 0, -1):
            sa_right = add(sa_right, s[i].box)
            count += s[i].size
            rc[i] = surface(sa_right) * float(count)
            rb[i] = sa_right
        count += s[0].size
        best = [surface(box) * float(count), (s, box, depth), None]
        count = s[0].size
        sa_left = s[0].box
        for i in range(1, n):
            cost = rc[i] + surface(sa_left) * float(count)
            if cost < best[0]:
                best = [cost, (s[:i], sa_left, depth), (s[i:], rb[i], depth)]
            sa_left = add(sa_left, s[i].box)
            count += s[i].size
        return best

    def sweep(cut):
        nodes, box, depth = cut
        a = sorted(nodes, key=lambda n: n.bc[0])
        s2 = sorted(a, key=lambda n: n.bc[1])
        xs = min_cost(a, box, depth)
        ys = min_cost(s2, box, depth)
        if xs[0] < ys[0]:
            s2 = sorted(s2, key=lambda n: n.bc[2])
            zs = min_cost(s2, box, depth)
            return (xs if xs[0] < zs[0] else zs)[1:]
        a = sorted(a, key=lambda n: n.bc[2])
        zs = min_cost(a, box, depth)
        return (ys if ys[0] < zs[0] else zs)[1:]

    def adopt(n):
        if isinstance(n, Out):
            return n
        if n.leaf:
            return Out(True, n.box, prims=list(n.prims))
        return make_leaf(n.box, [n])

    def build(cut):
        nodes, box, depth = cut
        if len(nodes) <= 1:
            return adopt(nodes[0])
        cuts = [cut]
        while len(cuts) < bf:
            mx, mi = 0, 0
            for i, c in enumerate(cuts):
                if len(c[0]) > mx:
                    mx, mi = len(c[0]), i
            if mx <= 1:
                break
            cost[0] += mx
            left, right = sweep(cuts[mi])
            if right is not None:
                cuts[mi] = refined(left)
                cuts.append(refined(right))
            else:
                cuts[mi] = ([make_leaf(left[1], left[0])], None, 0)
        return Out(False, box, kids=[build(c) for c in cuts])

    # findInitialCut, FIFO order
    q = deque([root])
    counter = 0
    cut = []
    t0 = thr(0)
    while q:
        n = q.popleft()
        if n.leaf:
            cut.append(n)
        elif surface(n.box) > t0:
            counter += len(n.kids) - 1
            if counter >= MAX_CUT_SIZE:
                cut.append(n)
            else:
                q.extend(n.kids)
        else:
            cut.append(n)
    cost[0] += len(cut)
    out = build((cut, root.box, 1))
    if stats is not None:
        stats["build_cost"] = cost[0]
    return out


def export(root):
    kind, count, box, prims = [], [], [], []
    st = [root]
    while st:
        n = st.pop()
        kind.append(1 if n.leaf else 0)
        box.append(n.box)
        if n.leaf:
            count.append(len(n.prims))
            prims.extend(n.prims)
        else:
            count.append(len(n.kids))
            st.extend(reversed(n.kids))
    return (np.asarray(kind, np.int8), np.asarray(count, np.int32), np.asarray(box, np.float64),
            np.asarray(prims, np.int32))
