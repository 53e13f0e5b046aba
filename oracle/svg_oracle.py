"""A Python restatement of lyon_extra's PathParser (crates/extra/src/parser.rs:138-490) and of
the arc conversion it uses (crates/geom/src/arc.rs:58-138, 668-703) — TEST INFRASTRUCTURE ONLY,
the checker of the library's SVG parser. f32 arithmetic through numpy; the f32 math functions
sqrtf and fmodf are the C library's (exact), cos, sin and tan are evaluated in f64 and rounded
once, as the library's parser does (lyon takes them from the platform's f32 libm); `angle_from_x_axis` is euclid 0.22.9's `fast_atan2` (the published polynomial
of math.stackexchange question 1098487, answer 1105038), in f32 as lyon evaluates it.

parse(src, num_attributes, stop_at) -> (verbs, points, widths, error) with error None or
(kind, line, column), kind one of "number", "flag", "command", "missing_move_to".
"""

from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _name in ("cosf", "sinf", "tanf", "sqrtf"):
    getattr(_libm, _name).restype = ctypes.c_float
    getattr(_libm, _name).argtypes = [ctypes.c_float]
for _name in ("fmodf",):
    getattr(_libm, _name).restype = ctypes.c_float
    getattr(_libm, _name).argtypes = [ctypes.c_float, ctypes.c_float]

f32 = np.float32
PI = f32(math.pi)

BEGIN, LINE, QUAD, CUBIC, CLOSE, END = 3, 0, 1, 2, 4, 5


class _Src:
    def __init__(self, s):
        self.s = s
        self.i = 0
        if s:
            self.cur = s[0]
            self.i = 1
            self.fin = False
        else:
            self.cur = " "
            self.fin = True
        self.line = 1 if self.cur == "\n" else 0
        self.col = 0

    def adv(self):
        if self.fin:
            return
        if self.i >= len(self.s):
            self.cur = "~"
            self.fin = True
            return
        c = self.s[self.i]
        self.i += 1
        if c == "\n":
            self.cur = "\n"
            self.line += 1
            self.col = -1
        else:
            self.cur = c
            self.col += 1

    def skip_ws(self):
        while not self.fin and (self.cur.isspace() or self.cur == ","):
            self.adv()


class _Err(Exception):
    def __init__(self, kind, line, col):
        self.kind, self.line, self.col = kind, line, col


class _Out:
    def __init__(self):
        self.verbs, self.points, self.widths = [], [], []
        self.first, self.first_w = (f32(0), f32(0)), f32(0)

    def pt(self, p, w):
        self.points.append((f32(p[0]), f32(p[1])))
        self.widths.append(f32(w))

    def begin(self, p, w):
        self.first, self.first_w = p, w
        self.pt(p, w)
        self.verbs.append(BEGIN)

    def line(self, p, w):
        self.pt(p, w)
        self.verbs.append(LINE)

    def quad(self, c, p, w):
        self.pt(c, 0)
        self.pt(p, w)
        self.verbs.append(QUAD)

    def cubic(self, c1, c2, p, w):
        self.pt(c1, 0)
        self.pt(c2, 0)
        self.pt(p, w)
        self.verbs.append(CUBIC)

    def end(self, close):
        if close:
            self.pt(self.first, self.first_w)
        self.verbs.append(CLOSE if close else END)


_C = {math.sqrt: _libm.sqrtf}


def _fn(f, x):
    # cos, sin and tan: f64 evaluation rounded once, as the library's parser evaluates them (lyon
    # takes them from the platform's f32 libm, within an ulp of these); sqrt is exact in f32.
    if f in _C:
        return f32(_C[f](float(x)))
    return f32(f(float(x)))


def decimal_to_f32(text: str):
    """Rust's f32::from_str: the decimal rounded to the nearest f32, ties to even, computed
    exactly with rationals (a conversion through f64 would round twice)."""
    import struct
    from fractions import Fraction
    v = Fraction(text)
    neg = text.lstrip().startswith("-")
    if v == 0:
        return f32(-0.0) if neg else f32(0.0)
    a = abs(v)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    e = max(e, -126)                       # subnormals share the smallest exponent
    scaled = a * Fraction(2) ** (23 - e)   # the 24-bit significand, with a fraction
    m = scaled.numerator // scaled.denominator
    rem = scaled - m
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and m % 2 == 1):
        m += 1
    if m == 1 << 24:
        m >>= 1
        e += 1
    if e > 127:
        r = float("inf")
    else:
        r = float(Fraction(m) * Fraction(2) ** (e - 23))
    r = struct.unpack("<f", struct.pack("<f", r))[0]  # exact: r is an f32 value
    return f32(-r if neg else r)


def _atan2(y, x):
    # euclid's Trig::fast_atan2 for f32: numpy float32 scalars round every operation to f32.
    y, x = f32(y), f32(x)
    xa, ya = abs(x), abs(y)
    with np.errstate(invalid="ignore", divide="ignore"):
        a = f32(min(xa, ya) / max(xa, ya))
    s = a * a
    r = ((f32(-0.0464964749) * s + f32(0.15931422)) * s - f32(0.327622764)) * s * a + a
    if ya > xa:
        r = f32(math.pi / 2) - r
    if x < 0:
        r = PI - r
    if y < 0:
        r = -r
    return f32(r)


def _fmod(a, b):
    return f32(_libm.fmodf(float(a), float(b)))


def _rot(a, v):
    s, c = _fn(math.sin, a), _fn(math.cos, a)
    return (v[0] * c - v[1] * s, v[0] * s + v[1] * c)


def _arc_quads(frm, to, rx, ry, xrot, large, sweep):
    rx, ry = abs(rx), abs(ry)
    two_pi = f32(2) * PI
    xr = _fmod(xrot, two_pi)
    cp, sp = _fn(math.cos, xr), _fn(math.sin, xr)
    hdx, hdy = (frm[0] - to[0]) / f32(2), (frm[1] - to[1]) / f32(2)
    hsx, hsy = (frm[0] + to[0]) / f32(2), (frm[1] + to[1]) / f32(2)
    px, py = cp * hdx + sp * hdy, -sp * hdx + cp * hdy
    rf = px * px / (rx * rx) + py * py / (ry * ry)
    if rf > 1:
        sc = _fn(math.sqrt, rf)
        rx, ry = rx * sc, ry * sc
    rxry, rxpy, rypx = rx * ry, rx * py, ry * px
    ssq = rxpy * rxpy + rypx * rypx
    sign_coe = f32(-1) if large == sweep else f32(1)
    coe = sign_coe * _fn(math.sqrt, abs((rxry * rxry - ssq) / ssq))
    tcx = coe * rxpy / ry
    tcy = -coe * rypx / rx
    cx, cy = cp * tcx - sp * tcy + hsx, sp * tcx + cp * tcy + hsy
    sv = ((px - tcx) / rx, (py - tcy) / ry)
    ev = ((-px - tcx) / rx, (-py - tcy) / ry)
    start = _atan2(sv[1], sv[0])
    sweep_a = _fmod(_atan2(ev[1], ev[0]) - start, two_pi)
    if sweep and sweep_a < 0:
        sweep_a += two_pi
    elif not sweep and sweep_a > 0:
        sweep_a -= two_pi
    sign = f32(-1) if np.signbit(sweep_a) else f32(1)
    sw = min(abs(sweep_a), PI * f32(2))
    n_steps = f32(math.ceil(float(sw / (PI / f32(4)))))
    step = sw / n_steps * sign
    t0 = f32(0)
    dt = f32(1) / n_steps
    alpha = _fn(math.tan, step * f32(0.5))
    out = []
    n = int(n_steps)
    for i in range(n):
        a1 = start + step * f32(i)
        a2 = start + step * f32(i + 1)
        v1 = _rot(xrot, (rx * _fn(math.cos, a1), ry * _fn(math.sin, a1)))
        v2 = _rot(xrot, (rx * _fn(math.cos, a2), ry * _fn(math.sin, a2)))
        fp = (cx + v1[0], cy + v1[1])
        tp = (cx + v2[0], cy + v2[1])
        tg = _rot(xrot, (-rx * _fn(math.sin, a1), ry * _fn(math.cos, a1)))
        ctrl = (fp[0] + tg[0] * alpha, fp[1] + tg[1] * alpha)
        t1 = f32(1) if i + 1 == n else t0 + dt
        out.append((ctrl, tp, t1))
        t0 = t1
    return out


def parse(src: str, num_attributes: int = 0, stop_at=None):
    s = _Src(src)
    o = _Out()
    st = {"cur": (f32(0), f32(0)), "attr": f32(0), "need_end": False}

    def number():
        s.skip_ws()
        line, col = s.line, s.col
        buf = ""
        if s.cur == "-":
            buf += "-"
            s.adv()
        m = 0
        while s.cur.isascii() and s.cur.isdigit():
            buf += s.cur
            s.adv()
            m += 1
        if s.cur == ".":
            buf += "."
            s.adv()
            while s.cur.isascii() and s.cur.isdigit():
                buf += s.cur
                s.adv()
                m += 1
        ok = True
        if s.cur in "eE":
            buf += s.cur
            s.adv()
            if s.cur == "-":
                buf += "-"
                s.adv()
            e = 0
            while s.cur.isascii() and s.cur.isdigit():
                buf += s.cur
                s.adv()
                e += 1
            ok = e > 0
        if m == 0 or not ok:
            raise _Err("number", line, col)
        return decimal_to_f32(buf)

    def flag():
        s.skip_ws()
        if s.cur in "01":
            v = s.cur == "1"
            s.adv()
            return v
        raise _Err("flag", s.line, s.col)

    def attributes():
        if num_attributes:
            st["attr"] = number()

    def point(rel):
        x, y = number(), number()
        if rel:
            x, y = x + st["cur"][0], y + st["cur"][1]
        return (x, y)

    def endpoint(rel):
        p = point(rel)
        st["cur"] = p
        attributes()
        return p

    def smooth(prev):
        c = st["cur"]
        return c if prev is None else (c[0] + (c[0] - prev[0]), c[1] + (c[1] - prev[1]))

    err = None
    try:
        first = (f32(0), f32(0))
        need_start = False
        pc = pq = None
        implicit = "M"
        s.skip_ws()
        while not s.fin:
            cmd = s.cur
            cl, cc = s.line, s.col
            if stop_at is not None and cmd == stop_at:
                break
            if cmd.isascii() and cmd.isalpha():
                s.adv()
            else:
                cmd = implicit
            if need_start and cmd not in "mM":
                raise _Err("missing_move_to", cl, cc)
            rel = cmd.islower()
            if cmd in "lL":
                o.line(endpoint(rel), st["attr"])
            elif cmd in "hH":
                x = number()
                if rel:
                    x = x + st["cur"][0]
                st["cur"] = (x, st["cur"][1])
                attributes()
                o.line(st["cur"], st["attr"])
            elif cmd in "vV":
                y = number()
                if rel:
                    y = y + st["cur"][1]
                st["cur"] = (st["cur"][0], y)
                attributes()
                o.line(st["cur"], st["attr"])
            elif cmd in "qQ":
                c = point(rel)
                t = endpoint(rel)
                pq = c
                o.quad(c, t, st["attr"])
            elif cmd in "tT":
                c = smooth(pq)
                t = endpoint(rel)
                pq = c
                o.quad(c, t, st["attr"])
            elif cmd in "cC":
                c1, c2 = point(rel), point(rel)
                t = endpoint(rel)
                pc = c2
                o.cubic(c1, c2, t, st["attr"])
            elif cmd in "sS":
                c1 = smooth(pc)
                c2 = point(rel)
                t = endpoint(rel)
                pc = c2
                o.cubic(c1, c2, t, st["attr"])
            elif cmd in "aA":
                pa = st["attr"]
                frm = st["cur"]
                rx, ry, xr = number(), number(), number()
                la, sw = flag(), flag()
                t = endpoint(rel)
                eps = f32(1.1920929e-07)
                if abs(rx) <= eps or abs(ry) <= eps or (frm[0] == t[0] and frm[1] == t[1]):
                    o.line(t, st["attr"])
                else:
                    ea = st["attr"]
                    for c, tp, t1 in _arc_quads(frm, t, rx, ry, xr * (PI / f32(180)), la, sw):
                        o.quad(c, tp, pa * (f32(1) - t1) + ea * t1)
            elif cmd in "mM":
                if st["need_end"]:
                    o.end(False)
                    st["need_end"] = False
                t = endpoint(rel)
                first = t
                o.begin(t, st["attr"])
                st["need_end"] = True
                need_start = False
            elif cmd in "zZ":
                o.end(True)
                st["cur"] = first
                st["need_end"] = False
                need_start = True
            else:
                raise _Err("command", cl, cc)
            if cmd in "cCsS":
                pq = None
            elif cmd in "qQtT":
                pc = None
            else:
                pc = pq = None
            implicit = {"m": "l", "M": "L", "z": "m", "Z": "M"}.get(cmd, cmd)
            s.skip_ws()
    except _Err as e:
        err = (e.kind, e.line, e.col)
    if st["need_end"]:
        o.end(False)
    pts = np.array(o.points, np.float32).reshape(-1, 2)
    return (np.array(o.verbs, np.uint8), pts, np.array(o.widths, np.float32), err)
