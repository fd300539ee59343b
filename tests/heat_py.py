"""A pure-Python restatement of the reference's heat-map renderer, used only to
cross-check the C oracle on small inputs: pixel-centre camera rays
(camera.go:53-97), BVH.traversalSteps (bvh.go:21-44) with aabb.intersected
(bounding.go:53-90) and Triangle.intersected (primitive.go:172-208), and
DefaultTraversalCountShader (render.go:250-257).  Trees come from an oracle
pre-order export (tests/phr_py.parse)."""
import math

APPROX_THRESH = 1e-7  # util.go


def sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def mul(a, s):
    return (a[0] * s, a[1] * s, a[2] * s)


def dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def unit(a):
    n = math.sqrt(dot(a, a))
    return (a[0] / n, a[1] / n, a[2] / n)


def camera(cam):
    """NewCamera + SetTransformation (camera.go:53-92): origin, lower-left corner, horizontal, vertical."""
    vh = 2.0 * math.tan((cam["fov"] * (math.pi / 180)) / 2)
    vw = cam["aspect"] * vh
    w = unit(sub(cam["look_from"], cam["look_at"]))
    u = unit(cross(cam["up"], w))
    v = cross(w, u)
    o = tuple(float(x) for x in cam["look_from"])
    hor, ver = mul(u, vw), mul(v, vh)
    llc = sub(sub(sub(o, mul(hor, 0.5)), mul(ver, 0.5)), w)
    return o, llc, hor, ver


def inverse(d):  # math.go:70-72; Go's 1/0 is a signed infinity
    return tuple((1.0 / x) if x != 0 else math.copysign(math.inf, x) for x in d)


def box_hit(b, o, inv, sign, tmin, tmax):
    lo, hi = b[:3], b[3:]

    def bnd(s, k):
        return hi[k] if s else lo[k]

    txmin = (bnd(sign[0], 0) - o[0]) * inv[0]
    txmax = (bnd(1 - sign[0], 0) - o[0]) * inv[0]
    tymin = (bnd(sign[1], 1) - o[1]) * inv[1]
    tymax = (bnd(1 - sign[1], 1) - o[1]) * inv[1]
    if txmin > tymax or tymin > txmax:
        return False
    if tymin > txmin:
        txmin = tymin
    if tymax < txmax:
        txmax = tymax
    tzmin = (bnd(sign[2], 2) - o[2]) * inv[2]
    tzmax = (bnd(1 - sign[2], 2) - o[2]) * inv[2]
    if txmin > tzmax or tzmin > txmax:
        return False
    if tzmin > txmin:
        txmin = tzmin
    if tzmax < txmax:
        txmax = tzmax
    return not (txmax < tmin or txmin > tmax)


def tri_t(tri, o, d, tmin, tmax):
    v0, v1, v2 = tri[0:3], tri[3:6], tri[6:9]
    e1, e2 = sub(v1, v0), sub(v2, v0)
    pvec = cross(d, e2)
    det = dot(e1, pvec)
    if abs(det) <= APPROX_THRESH:
        return None
    inv_det = 1 / det
    tvec = sub(o, v0)
    u = dot(tvec, pvec) * inv_det
    if u < 0 or u > 1:
        return None
    qvec = cross(tvec, e1)
    v = dot(d, qvec) * inv_det
    if v < 0 or u + v > 1:
        return None
    t = dot(e2, qvec) * inv_det
    if t < tmin or t > tmax:
        return None
    return t


def traversal_steps(root, tris, o, d, tmin, tmax):
    inv = inverse(d)
    sign = [1 if x < 0 else 0 for x in inv]
    stack = [root]
    count = 0
    t_hit = tmax
    while stack:
        n = stack.pop()
        if not box_hit(n.box, o, inv, sign, tmin, t_hit):
            continue
        if n.leaf:
            for p in n.prims:
                t = tri_t(tris[p], o, d, tmin, t_hit)
                if t is not None:
                    t_hit = t
        else:
            stack.extend(n.kids)
            count += 1
    return count


def shade(count, threshold):
    if count > threshold:
        return (count / threshold * 2, 0.0, 0.0)
    f = count / (threshold * 1.25)
    return (0.0, f, 1 - f)


def heatmap(root, tris, cam, width, height, threshold):
    o, llc, hor, ver = camera(cam)
    counts, rgb = [], []
    for y in range(height):
        for x in range(width):
            u, v = x / (width - 1), y / (height - 1)
            d = sub(add(add(llc, mul(hor, u)), mul(ver, v)), o)
            c = traversal_steps(root, tris, o, d, 0.001, 1.7976931348623157e308)
            counts.append(c)
            rgb.append(shade(c, threshold))
    return counts, rgb
