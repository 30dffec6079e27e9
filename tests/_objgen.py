"""Seeded OBJ files that put the reference loader's parsing edge cases
(src/symvox/scene.cpp:98-233, buildTriVector :394-416) on both sides of the
threaded ingest's cut points, and a restatement of those parsing rules.
Shared by tests/test_obj_ingest.py and tests/golden/make_golden.py."""
import ctypes
import ctypes.util

import numpy as np

_libc = ctypes.CDLL(ctypes.util.find_library("c"))


def _scan_floats(s):
    p = (ctypes.c_float * 3)()
    n = _libc.sscanf(s, b"%f %f %f", ctypes.byref(p, 0), ctypes.byref(p, 4), ctypes.byref(p, 8))
    return n, list(p)


def _scan_index(s):
    iv, iN = ctypes.c_int(0), ctypes.c_int(0)
    n = _libc.sscanf(s, b"%d//%d", ctypes.byref(iv), ctypes.byref(iN))
    return n, iv.value


def reference_parse(data):
    """The reference's loader rules: fgets records of at most 9999 bytes,
    'v' records read with "%f %f %f", 'f' records split on ' ' with the last
    token's final byte dropped, corners read with "%d//%d", negative indices
    counted back from the vertices read so far, a second triangle (tokens
    2, 3, 0) only when more than four tokens, a corner without an index keeps
    the previous triangle's, triangles with an index out of range dropped."""
    verts, idx = [], []
    lo, hi = [np.float32(np.finfo(np.float32).max)] * 3, [np.float32(-np.finfo(np.float32).max)] * 3
    pos = 0
    while pos < len(data):
        span = data[pos:pos + 9999]
        nl = span.find(b"\n")
        rec = span[:nl + 1] if nl >= 0 else span
        pos += len(rec)
        line = rec.split(b"\0")[0]
        if line[:1] == b"v":
            if line[1:2] in (b"n", b"t"):
                continue
            n, p = _scan_floats(line[1:])
            if n != 3:
                continue
            p = [np.float32(x) for x in p]
            for k in range(3):
                if p[k] < lo[k]:
                    lo[k] = p[k]
                if p[k] > hi[k]:
                    hi[k] = p[k]
            verts.append(p)
        elif line[:1] == b"f":
            tok = [t for t in line[1:].split(b" ") if t]
            if not tok:
                continue
            tok[-1] = tok[-1][:-1]
            if len(tok) < 3:
                continue

            def corner(t, prev):
                n, iv = _scan_index(t)
                if iv < 0:
                    iv = len(verts) + iv + 1
                return (iv - 1) % (1 << 64) if n >= 1 else prev

            t0 = [corner(tok[i], (1 << 64) - 1) for i in range(3)]
            idx.append(t0)
            if len(tok) > 4:
                idx.append([corner(tok[(i + 2) % 4], t0[i]) for i in range(3)])
    nv = len(verts)
    tris = [sum((verts[i] for i in t), []) for t in idx if all(i < nv for i in t)]
    return np.array(tris, np.float32).reshape(-1, 9), np.array(lo + hi, np.float32)


# face records with fewer than three space-separated tokens: the reference's
# loader reads past its token list on them (it crashes), so the files that
# are run through the reference itself leave them out
SHORT_FACES = (b"f\n", b"f 1 2\n", b"f\t1\t2\t3\n")


def edge_lines(rng, nv, reference_safe=False):
    """Records covering the rules' edge cases, given nv vertices so far."""
    a, b, c = (int(x) for x in rng.integers(1, nv + 1, 3))
    while True:
        line = _edge_line(rng, nv, a, b, c)
        if not (reference_safe and line in SHORT_FACES):
            return line


def _edge_line(rng, nv, a, b, c):
    return rng.choice([
        b"f %d %d %d\n" % (a, b, c),
        b"f %d %d %d\r\n" % (a, b, c),
        b"f -1 -2 -3\n",
        b"f %d %d %d %d \n" % (a, b, c, a),          # five tokens: a second triangle
        b"f %d %d %d %d\n" % (a, b, c, a),           # four tokens: one triangle
        b"f %d/1/2 %d/3/4 %d/5/6\n" % (a, b, c),
        b"f %d//1 %d//2 %d//3\n" % (a, b, c),
        b"f  %d   %d %d\n" % (a, b, c),
        b"f x %d %d %d \n" % (a, b, c),              # a corner without an index
        b"f 0 %d %d\n" % (b, c),                      # index 0: dropped
        b"f %d %d %d\n" % (a, b, nv + 1000),          # out of range: dropped
        b"f\n", b"f 1 2\n", b"f\t1\t2\t3\n",
        b"vn 0 1 0\n", b"vt 0.5 0.5\n", b"v 1 2\n", b"vp 1 2 3\n", b"# comment\n", b"\n",
        b"v\t0.25\t0.5\t0.75\n", b"v -0 0 -0\n", b"v 1e-3 2.5e+1 -7\n",
        # numbers outside the plain-decimal fast path, decided by the C library
        b"v 16777217 16777219 0.1\n", b"v 1.000000059604644775390625 2 3\n", b"v 1e400 0 0\n",
        b"v 1e-50 2e-39 3\n", b"v 0x1p3 1 2\n", b"v nan 1 2\n", b"v inf -inf 1\n", b"v 1.5x 2 3\n",
        b"v 1.5e 2 3\n", b"v .5 5. -.25\n", b"v +1 +2.5 -3E2\n", b"v 0.123456789012345678901234 1 2\n",
        b"v 3.4028235e38 -3.4028236e38 1\n", b"v 1 2 3 4\n", b"v 1,2 3 4\n", b"v 7e22 7e23 1e-22\n",
        b"f +%d %d -0\n" % (a, b), b"f 99999999999 %d %d\n" % (b, c), b"f %d// %d//x %d\n" % (a, b, c),
    ])


def make_obj(seed, n_lines, long_lines=True, final_newline=True, reference_safe=False):
    rng = np.random.default_rng(seed)
    out, nv = [], 0
    for _ in range(n_lines):
        r = rng.random()
        if r < 0.45 or nv < 3:
            x = rng.random(3) * 2 - 0.5
            out.append(b"v %.9g %.9g %.9g\n" % tuple(x))
            nv += 1
        elif r < 0.9:
            a, b, c = (int(x) for x in rng.integers(1, nv + 1, 3))
            out.append(b"f %d %d %d\n" % (a, b, c))
        elif r < 0.999 or not long_lines:
            line = edge_lines(rng, nv, reference_safe)
            nv += line[:1] == b"v" and line[1:2] not in (b"n", b"t") and _scan_floats(line[1:])[0] == 3
            out.append(line)
        else:
            # a record longer than the reference's 9999-byte line buffer:
            # its continuation is read as a record of its own
            pad = b"#" + b"x" * 9997
            out.append(pad + b"v 0.125 0.25 0.375\n")
            nv += 1
    data = b"".join(out)
    if not final_newline:
        data += b"f 1 2 34"
    return data
