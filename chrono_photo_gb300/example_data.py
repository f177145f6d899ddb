"""Seeded synthetic frame stacks (the reference's create-test-data, src/util/
create_example_data.rs, draws unseeded noise; these generators are reproducible).

Background: a smooth gradient g_c(x, y) = a_c + b_c*x/W + d_c*y/H plus i.i.d. Gaussian noise,
rounded half away from zero and clamped to [0, 255]. Foreground: solid disks of a uniformly
drawn colour moving along straight (or sinusoidal) paths, one position per frame.
Frames are uint8 [n, h, w, 3], frame-major, as the compositing kernels read them.
"""
import numpy as np


def _round_clamp(x):
    return np.clip(np.floor(x + 0.5), 0, 255).astype(np.uint8)


class Disk:
    def __init__(self, rng, w, h, n, rmin, rmax, path="line"):
        self.r = float(rng.uniform(rmin, rmax))
        self.color = rng.integers(0, 256, size=3).astype(np.float32)
        self.x0, self.y0 = rng.uniform(0, w), rng.uniform(0, h)
        self.x1, self.y1 = rng.uniform(0, w), rng.uniform(0, h)
        self.path = path
        self.amp = rng.uniform(0.1, 0.3) * h
        self.periods = rng.uniform(1, 3)
        self.n = max(n - 1, 1)

    def center(self, i):
        t = i / self.n
        x = self.x0 + (self.x1 - self.x0) * t
        y = self.y0 + (self.y1 - self.y0) * t
        if self.path == "sine":
            y = self.y0 + self.amp * np.sin(2 * np.pi * self.periods * t)
        return x, y


def _background(rng, w, h):
    a = rng.uniform(40, 160, size=3)
    b = rng.uniform(-40, 40, size=3)
    d = rng.uniform(-40, 40, size=3)
    xs = (np.arange(w, dtype=np.float32) / w)[None, :, None]
    ys = (np.arange(h, dtype=np.float32) / h)[:, None, None]
    return (a[None, None, :] + b[None, None, :] * xs + d[None, None, :] * ys).astype(np.float32)


def _texture(rng, w, h, k=8):
    xs = np.arange(w, dtype=np.float32)[None, :]
    ys = np.arange(h, dtype=np.float32)[:, None]
    t = np.zeros((h, w), np.float32)
    for _ in range(k):
        fx, fy = rng.uniform(0.04, 0.35, size=2)
        ph = rng.uniform(0, 2 * np.pi)
        amp = rng.uniform(6, 16)
        t += amp * np.sin(fx * xs + fy * ys + ph).astype(np.float32)
    return t[..., None]


def stack(n, w, h, sigma=3.0, n_disks=1, rmin=20, rmax=20, seed=1, path="line", drift=0.0,
          texture=False, shifts=None, out=None):
    """n frames of w x h RGB. drift: per-frame gain uniform in [1-drift, 1+drift] on the
    background; shifts: per-frame integer (dx, dy) translation of the background;
    out: optional preallocated uint8 [n, h, w, 3] (e.g. pinned host memory)."""
    rng = np.random.default_rng(seed)
    base = _background(rng, w, h)
    pad = 0
    if shifts is not None:
        pad = int(np.max(np.abs(shifts))) + 1
    if texture:
        bw, bh = w + 2 * pad, h + 2 * pad
        big = _background(rng, bw, bh) + _texture(rng, bw, bh)
    else:
        big = None
    disks = [Disk(rng, w, h, n, rmin, rmax, path) for _ in range(n_disks)]
    gains = rng.uniform(1 - drift, 1 + drift, size=n) if drift else np.ones(n)
    frames = out if out is not None else np.empty((n, h, w, 3), np.uint8)
    yy = np.arange(h, dtype=np.float32)[:, None]
    xx = np.arange(w, dtype=np.float32)[None, :]
    for i in range(n):
        if big is not None:
            dx, dy = (shifts[i] if shifts is not None else (0, 0))
            bg = big[pad + dy:pad + dy + h, pad + dx:pad + dx + w]
        else:
            bg = base
        f = bg * np.float32(gains[i]) + rng.standard_normal((h, w, 3), dtype=np.float32) * sigma
        for dsk in disks:
            cx, cy = dsk.center(i)
            x0, x1 = max(int(cx - dsk.r) - 1, 0), min(int(cx + dsk.r) + 2, w)
            y0, y1 = max(int(cy - dsk.r) - 1, 0), min(int(cy + dsk.r) + 2, h)
            if x0 >= x1 or y0 >= y1:
                continue
            m = (xx[:, x0:x1] - cx) ** 2 + (yy[y0:y1] - cy) ** 2 <= dsk.r ** 2
            f[y0:y1, x0:x1][m] = dsk.color
        frames[i] = _round_clamp(f)
    return frames


# The named workloads: frame counts, sizes and content of each configuration.
def small_stack(seed=1, scale=1):
    """16 frames of 640x480 (sigma 3, one r=20 disk on a straight line)."""
    return stack(16, 640 // scale, 480 // scale, sigma=3, n_disks=1, rmin=20 / scale,
                 rmax=20 / scale, seed=seed)


def hd_stack(seed=2, n=64, w=1920, h=1080, out=None):
    """64 frames of 1920x1080 (sigma 4, three disks r in [10, 40] on their own lines)."""
    return stack(n, w, h, sigma=4, n_disks=3, rmin=10, rmax=40, seed=seed, out=out)


def video_stack(seed=3, n=300, w=1920, h=1080, out=None):
    """300 frames of 1920x1080 with +-5% brightness drift and one disk on a sine path."""
    return stack(n, w, h, sigma=4, n_disks=1, rmin=30, rmax=30, seed=seed, path="sine",
                 drift=0.05, out=out)


def shake_stack(seed=5, n=100, w=6000, h=4000, max_shift=12, n_disks=5, rmin=20, rmax=60):
    """Textured background translated per frame by U[-12, 12]^2, 5 disks. Returns
    (frames, shifts): frame i shows the background window at shifts[i], so the shake offsets
    of frame i relative to frame 0 are shifts[0] - shifts[i]."""
    rng = np.random.default_rng(seed + 1000)
    shifts = rng.integers(-max_shift, max_shift + 1, size=(n, 2))
    frames = stack(n, w, h, sigma=3, n_disks=n_disks, rmin=rmin, rmax=rmax, seed=seed,
                   texture=True, shifts=shifts)
    return frames, shifts


def job_specs(seed=4, count=512):
    """Mixed jobs: N ~ U{8..128}, resolution ~ U{320x240, 1280x720, 1920x1080, 4000x3000},
    outlier mode ~ U{extreme, average, first, last}, own generator seed per job."""
    rng = np.random.default_rng(seed)
    res = [(320, 240), (1280, 720), (1920, 1080), (4000, 3000)]
    modes = ["extreme", "average", "first", "last"]
    jobs = []
    for j in range(count):
        n = int(rng.integers(8, 129))
        w, h = res[int(rng.integers(0, 4))]
        jobs.append(dict(n=n, w=w, h=h, outlier=modes[int(rng.integers(0, 4))], seed=seed * 100000 + j))
    return jobs


def _png_chunk(kind, body):
    import struct
    import zlib
    return (struct.pack(">I", len(body)) + kind + body +
            struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF))


def encode_png(img, level=6):
    """PNG bytes of a uint8 [h, w, c] image (c = 1, 3 or 4), every scanline Paeth-filtered
    (filter type 4, the usual choice of encoders for photographs), zlib at `level`."""
    import struct
    import zlib
    h, w, c = img.shape
    x = img.reshape(h, w * c).astype(np.int16)
    a = np.zeros_like(x)
    a[:, c:] = x[:, :-c]
    b = np.zeros_like(x)
    b[1:] = x[:-1]
    cc = np.zeros_like(x)
    cc[1:, c:] = x[:-1, :-c]
    p = a + b - cc
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - cc)
    pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, cc))
    rows = np.empty((h, w * c + 1), np.uint8)
    rows[:, 0] = 4
    rows[:, 1:] = ((x - pred) & 0xFF).astype(np.uint8)
    ihdr = struct.pack(">IIBBBBB", w, h, 8, {1: 0, 3: 2, 4: 6}[c], 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", ihdr) +
            _png_chunk(b"IDAT", zlib.compress(rows.tobytes(), level)) + _png_chunk(b"IEND", b""))


def write_pngs(frames, directory, level=6, threads=8):
    """Writes frames [n, h, w, c] as directory/frame_00000.png ... on a thread pool (zlib
    releases the interpreter lock); returns the paths in frame order."""
    import concurrent.futures as cf
    import os

    def one(i):
        path = os.path.join(directory, "frame_%05d.png" % i)
        with open(path, "wb") as f:
            f.write(encode_png(frames[i], level))
        return path
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, range(len(frames))))


def shake_stack_device(n, w, h, max_shift, seed):
    """Seeded shake stack generated on the CUDA device with torch (the host generator would
    take minutes at 100 x 6000x4000): gradient + 8 random-phase sinusoids, translated per frame
    by U[-s, s]^2, plus sigma-3 noise and 5 moving disks. Returns (uint8 [n, h, w, 3] device
    tensor, shifts); the shake offsets of frame i relative to frame 0 are shifts[0] - shifts[i]."""
    import torch
    rng = np.random.default_rng(seed)
    shifts = rng.integers(-max_shift, max_shift + 1, size=(n, 2))
    pad = max_shift + 1
    bw, bh = w + 2 * pad, h + 2 * pad
    dev = torch.device("cuda")
    xs = torch.arange(bw, device=dev, dtype=torch.float32)[None, :]
    ys = torch.arange(bh, device=dev, dtype=torch.float32)[:, None]
    a = rng.uniform(40, 160, size=3)
    b = rng.uniform(-40, 40, size=3)
    d = rng.uniform(-40, 40, size=3)
    tex = torch.zeros(bh, bw, device=dev)
    for _ in range(8):
        fx, fy = rng.uniform(0.04, 0.35, size=2)
        tex += float(rng.uniform(6, 16)) * torch.sin(float(fx) * xs + float(fy) * ys + float(rng.uniform(0, 6.283)))
    big = torch.stack([float(a[c]) + float(b[c]) * xs / bw + float(d[c]) * ys / bh + tex
                       for c in range(3)], dim=-1)
    # 16 spare bytes after the last frame: the kernels' 16-byte row copies may read past it
    flat = torch.zeros(n * h * w * 3 + 16, dtype=torch.uint8, device=dev)
    out = flat[:n * h * w * 3].view(n, h, w, 3)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    disks = [(rng.uniform(0, w), rng.uniform(0.4 * h, 0.6 * h), rng.uniform(0, w),
              rng.uniform(0.4 * h, 0.6 * h), rng.uniform(20, 60), rng.integers(0, 256, size=3))
             for _ in range(5)]
    for i in range(n):
        dx, dy = int(shifts[i][0]), int(shifts[i][1])
        f = big[pad + dy:pad + dy + h, pad + dx:pad + dx + w] + \
            3.0 * torch.randn((h, w, 3), generator=gen, device=dev)
        t = i / max(n - 1, 1)
        for (x0, y0, x1, y1, r, col) in disks:
            cx, cy = x0 + (x1 - x0) * t, y0 + (y1 - y0) * t
            xa, xb = max(int(cx - r) - 1, 0), min(int(cx + r) + 2, w)
            ya, yb = max(int(cy - r) - 1, 0), min(int(cy + r) + 2, h)
            if xa >= xb or ya >= yb:
                continue
            yy = torch.arange(ya, yb, device=dev, dtype=torch.float32)[:, None]
            xx = torch.arange(xa, xb, device=dev, dtype=torch.float32)[None, :]
            m = (xx - cx) ** 2 + (yy - cy) ** 2 <= r * r
            f[ya:yb, xa:xb][m] = torch.tensor([float(v) for v in col], device=dev)
        out[i] = torch.clamp(torch.floor(f + 0.5), 0, 255).to(torch.uint8)
    torch.cuda.synchronize()
    return out, shifts


def stack_device(n, w, h, sigma=3.0, n_disks=1, rmin=20, rmax=20, seed=1, path="line",
                 drift=0.0):
    """The `stack` recipe generated on the CUDA device with torch, for benchmark workloads too
    large for the host generator (300 frames of 1080p take about a minute in numpy): the same
    gradient background, per-frame gain, Gaussian noise and disks with the same seeded
    geometry, but the noise comes from torch's generator, so the frames are not the host
    generator's. Returns a uint8 [n, h, w, 3] device tensor whose storage has 16 spare bytes
    after the last frame (the kernels' 16-byte row copies may read up to there)."""
    import torch
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda")
    base = torch.from_numpy(_background(rng, w, h)).to(dev)
    disks = [Disk(rng, w, h, n, rmin, rmax, path) for _ in range(n_disks)]
    gains = rng.uniform(1 - drift, 1 + drift, size=n) if drift else np.ones(n)
    flat = torch.zeros(n * h * w * 3 + 16, dtype=torch.uint8, device=dev)
    out = flat[:n * h * w * 3].view(n, h, w, 3)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    for i in range(n):
        f = base * float(gains[i]) + float(sigma) * torch.randn((h, w, 3), generator=gen,
                                                                device=dev)
        for dsk in disks:
            cx, cy = dsk.center(i)
            x0, x1 = max(int(cx - dsk.r) - 1, 0), min(int(cx + dsk.r) + 2, w)
            y0, y1 = max(int(cy - dsk.r) - 1, 0), min(int(cy + dsk.r) + 2, h)
            if x0 >= x1 or y0 >= y1:
                continue
            yy = torch.arange(y0, y1, device=dev, dtype=torch.float32)[:, None]
            xx = torch.arange(x0, x1, device=dev, dtype=torch.float32)[None, :]
            m = (xx - float(cx)) ** 2 + (yy - float(cy)) ** 2 <= dsk.r ** 2
            f[y0:y1, x0:x1][m] = torch.tensor([float(v) for v in dsk.color], device=dev)
        out[i] = torch.clamp(torch.floor(f + 0.5), 0, 255).to(torch.uint8)
    torch.cuda.synchronize()
    return out


def video_stack_device(seed=3, n=300, w=1920, h=1080):
    """video_stack's recipe on the device (see stack_device)."""
    return stack_device(n, w, h, sigma=4, n_disks=1, rmin=30, rmax=30, seed=seed, path="sine",
                        drift=0.05)
