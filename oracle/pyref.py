"""Second, independent CPU restatement of the reference's per-pixel arithmetic in pure
Python with numpy float32 scalars (small cases only).

TEST INFRASTRUCTURE ONLY. It is written straight from the Rust sources, separately from
chrono_oracle.cpp, and the test suite checks the two against each other so that a
transcription slip in either shows up. Each function names the reference lines it follows.
"""
import math

import numpy as np

F = np.float32


def rround(x):
    """f32::round: half away from zero."""
    x = float(x)
    if math.isnan(x) or math.isinf(x):
        return F(x)
    return F(math.copysign(math.floor(abs(x) + 0.5), x))


def as_u8(x):
    """`f32 as u8`: saturating, NaN -> 0."""
    x = float(x)
    if math.isnan(x) or x <= 0:
        return 0
    if x >= 255:
        return 255
    return int(x)


def signum(w):
    w = F(w)
    if math.isnan(w):
        return w
    return F(-1.0) if math.copysign(1.0, float(w)) < 0 else F(1.0)


class Threshold:  # src/options.rs:189-231
    def __init__(self, absolute, mn, mx):
        mn, mx = F(mn), F(mx)
        self.absolute = absolute
        if absolute:
            self.min = F(mn * F(255))
            self.max = F(mx * F(255))
            self.scale = F(F(1) / F((mx - mn) * F(255)))
        else:
            self.min, self.max = mn, mx
            self.scale = F(F(1) / F(mx - mn))

    def blend_value(self, d):
        d = F(d)
        if d <= self.min:
            return F(0)
        if d >= self.max:
            return F(1)
        return F(F(d - self.min) * self.scale)


def fade_table(repeat, absolute, points):  # src/options.rs:69-139
    if not points:
        return lambda frame, total, off: F(1)
    offset = points[0][0]
    ln = points[-1][0] - offset
    values = [F(1)] * (ln + 1)
    idx = 0
    for i in range(ln + 1):
        f1, v1 = points[idx]
        f2, v2 = points[idx + 1]
        v1, v2 = F(v1), F(v2)
        frame = i + offset
        values[i] = F(v1 + F(F(F(v2 - v1) * F(frame - f1)) / F(f2 - f1)))
        if frame == f2:
            idx += 1

    def get(frame):
        i = frame - offset
        n = len(values)
        if 0 <= i < n:
            return values[i]
        if not repeat:
            return values[0] if i < 0 else values[n - 1]
        while i < 0:
            i += n
        return values[i % n]

    def fade(frame, total, off):  # src/chrono.rs:496-502
        return get(off + frame) if absolute else get(total - frame - 1)

    return fade


def quantile(d, q):  # src/chrono.rs:567-579
    pos = F(F(len(d) + 1) * F(q))
    p1 = int(pos) - 1
    frac = F(pos - F(math.trunc(float(pos))))
    if frac < F(0.001):
        return F(d[p1])
    if frac > F(0.999):
        return F(d[p1 + 1])
    return F(F(F(1) - frac) * F(d[p1]) + F(frac * F(d[p1 + 1])))


def median(d):  # src/chrono.rs:581-591
    n = len(d)
    if (n + 1) % 2 == 0:
        return F(d[(n + 1) // 2 - 1])
    i = (n + 1) // 2
    return F(F(0.5) * F(F(d[i - 1]) + F(d[i])))


def blend_into_u8(a, b, blend):  # src/color.rs:4-16
    if blend <= 0:
        return list(a)
    if blend >= 1:
        return list(b)
    return [as_u8(rround(F(F(x) + F(F(F(y) - F(x)) * blend)))) for x, y in zip(a, b)]


def calc_pixel(samples, thr, weights, background, outlier, fade, frame_offset, sample_idx=None,
               rng=None):
    """src/chrono.rs:208-494 for one pixel. samples: list of N tuples of C ints.
    Returns (pixel tuple, blend mask value, warning, detail dict)."""
    n = len(samples)
    c = len(samples[0])
    sample_idx = list(range(n)) if sample_idx is None else list(sample_idx)
    thr_sq = F(thr.min * thr.min)
    med = [F(0)] * 4
    iqr_inv = [F(0)] * 4
    q1s, q3s = [F(0)] * 4, [F(0)] * 4
    for i in range(c):
        if F(weights[i]) != 0:
            vals = sorted(samples[s][i] for s in sample_idx)
            if thr.absolute:
                med[i] = median(vals)
            else:
                q1, md, q3 = quantile(vals, 0.25), median(vals), quantile(vals, 0.75)
                med[i] = md
                q1s[i], q3s[i] = q1, q3
                iq = F(q3 - q1)
                if iq == 0:
                    iq = F(1)
                iqr_inv[i] = F(F(1) / iq)
    outl = []
    max_d, max_i = F(0), 0
    for s in range(n):
        d = F(0)
        for i in range(c):
            w = F(weights[i])
            if w != 0:
                diff = F(med[i] - F(samples[s][i]))
                if diff == 0:
                    term = F(0)
                elif thr.absolute:
                    t = F(w * diff)
                    term = F(signum(w) * F(t * t))
                else:
                    t = F(F(w * iqr_inv[i]) * diff)
                    term = F(signum(w) * F(t * t))
                d = F(d + term)
        if d >= thr_sq:
            outl.append((s, d))
            if d > max_d:
                max_d, max_i = d, s
    k = len(outl)
    warning = False
    bg_idx = -1
    if background == "average":
        mean = [F(0)] * 4
        for s in range(n):
            for i in range(c):
                mean[i] = F(mean[i] + F(samples[s][i]))
        mean = [F(m / F(n)) for m in mean]
        if k == 0:
            pix = [as_u8(rround(mean[i])) for i in range(c)]
        else:
            osum = [F(0)] * 4
            for s, _ in outl:
                for i in range(c):
                    osum[i] = F(osum[i] + F(samples[s][i]))
            ratio = F(F(n) / F(n - k))
            pix = [as_u8(rround(F(F(mean[i] * ratio) - F(osum[i] / F(n))))) for i in range(c)]
    elif background == "median":
        pix = [as_u8(rround(med[i])) for i in range(c)]
    elif background == "first":
        if k == 0:
            bg_idx = 0
        elif k == n:
            bg_idx, warning = 0, True
        else:
            ex = [s for s, _ in outl]
            bg_idx = next(i for i in range(n) if i not in ex)
        pix = list(samples[bg_idx])
    else:  # random, with the caller's draw function rng(m) -> [0, m)
        if k == 0 or k == n:
            bg_idx = rng(n)
            warning = k == n
        else:
            arr = list(range(n))
            cand = n
            for s, _ in outl:
                arr[s], arr[cand - 1] = arr[cand - 1], arr[s]
                cand -= 1
            bg_idx = arr[rng(cand)]
        pix = list(samples[bg_idx])
    detail = dict(median=med[:c], q1=q1s[:c], q3=q3s[:c], outliers=[s for s, _ in outl],
                  background=bg_idx)
    if k == 0:
        return tuple(pix), 0, warning, dict(detail, chosen=-1)
    if k == 1:
        s, d = outl[0]
        blend = F(fade(s, n, frame_offset) * thr.blend_value(F(np.sqrt(d))))
        pix = blend_into_u8(pix, samples[s], blend)
        return tuple(pix), as_u8(rround(F(blend * F(255)))), warning, dict(detail, chosen=s)
    if outlier in ("forward", "backward"):
        pf = [F(x) for x in pix]
        binv = F(1)
        order = outl if outlier == "forward" else list(reversed(outl))
        for s, d in order:
            b = F(fade(s, n, frame_offset) * thr.blend_value(F(np.sqrt(d))))
            if b <= 0:
                pass
            elif b >= 1:
                pf = [F(x) for x in samples[s]]
            else:
                pf = [F(a + F(F(F(x) - a) * b)) for a, x in zip(pf, samples[s])]
            binv = F(binv * F(F(1) - b))
        pix = [as_u8(rround(x)) for x in pf]
        return tuple(pix), as_u8(rround(F(F(F(1) - binv) * F(255)))), warning, dict(detail, chosen=-2)
    if outlier == "average":
        sums = [F(0)] * 4
        md = F(0)
        for s, d in outl:
            for i in range(c):
                sums[i] = F(sums[i] + F(samples[s][i]))
            md = F(md + F(np.sqrt(d)))
        sample = [as_u8(rround(F(sums[i] / F(k)))) for i in range(c)]
        si, dist = 0, F(md / F(k))
    else:
        if outlier == "first":
            si, d = outl[0]
        elif outlier == "last":
            si, d = outl[-1]
        else:
            si, d = max_i, max_d
        sample = list(samples[si])
        dist = F(np.sqrt(d))
    blend = F(fade(si, n, frame_offset) * thr.blend_value(dist))
    pix = blend_into_u8(pix, sample, blend)
    return tuple(pix), as_u8(rround(F(blend * F(255)))), warning, dict(detail, chosen=si)


def simple_pixel(samples, weights, darker, fade, frame_offset):
    """src/simple.rs:96-133 for one pixel."""
    n = len(samples)
    c = len(samples[0])
    ext = F(3.4028235e38) if darker else F(-3.4028235e38)
    out = [0] * c
    for s in range(n):
        v = F(0)
        for i in range(c):
            v = F(v + F(F(samples[s][i]) * F(weights[i])))
        if (v < ext) if darker else (v > ext):
            ext = v
            f = fade(s, n, frame_offset)
            if f > 0:
                out = list(samples[s]) if f >= 1 else blend_into_u8(out, samples[s], f)
    return tuple(out)
