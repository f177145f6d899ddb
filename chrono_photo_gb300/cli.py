"""Command-line front end with the reference's options: `python -m chrono_photo_gb300 ...`.

    chrono-photo (Rust)                                this module
    Cli / CliParsed (src/cli.rs:22-136, :140-236)      build_parser, parse_args
    options file `chrono-photo opts.chrono`            args_from_file (src/main.rs:33-43,
                                                       Cli::from_str src/cli.rs:238-258)
    FileLister + FrameRange (src/flist.rs)             list_files
    main / run_outliers / run_simple / create_video    run (src/main.rs:22-211)
    save_image (src/main.rs:519-570)                   api.save_image

Same flags, short forms and defaults (mode outlier, threshold abs/0.05/0.2, background
random, outlier extreme, quality 95, weights 1 1 1 1). The frames are decoded once (JPEG on
the GPU, PNG on host threads) and every composite runs on the GPU; the reference's
time-slice temp files do not exist here, so --temp-dir, --compression and --slice are
accepted and have no effect, as are --threads, --video-threads and --shake-threads (the
library sizes its own parallelism) and --wait. Errors the reference reports by panicking
exit with status 1 and the message.
"""
import argparse
import glob
import os
import re
import sys

import numpy as np

from . import api

OUTLIER_ONLY = ("output_blend", "threshold", "outlier", "background", "temp_dir", "sample",
                "slice", "compression")


class CliError(Exception):
    pass


def build_parser():
    ap = argparse.ArgumentParser(
        prog="chrono-photo",
        description="Combines images into a single chrono-photograph or chrono-video "
                    "(GB300 implementation of chrono-photo's compositing).")
    ap.add_argument("-p", "--pattern", required=True,
                    help="file search pattern (quote it on Unix systems)")
    ap.add_argument("-f", "--frames", help="frames to use of those matching: start/end/step")
    ap.add_argument("--video-in", help="frames per video frame: start/end/step")
    ap.add_argument("--video-out", help="range and step of video output frames: start/end/step")
    ap.add_argument("-o", "--output", required=True, help="path of the output file")
    ap.add_argument("--temp-dir", help="accepted for compatibility (no temp files are written)")
    ap.add_argument("--output-blend", help="path of the blend-mask image (mode outlier)")
    ap.add_argument("-m", "--mode", choices=["lighter", "darker", "outlier"])
    ap.add_argument("-t", "--threshold", help="(abs|rel)/<lower>[/<upper>]")
    ap.add_argument("-b", "--background", choices=["first", "random", "average", "median"])
    ap.add_argument("-l", "--outlier",
                    choices=["first", "last", "extreme", "average", "forward", "backward"])
    ap.add_argument("-c", "--compression", help="accepted for compatibility (no temp files)")
    ap.add_argument("-q", "--quality", type=int, help="JPEG output quality in percent (95)")
    ap.add_argument("-s", "--slice", help="accepted for compatibility (no temp files)")
    ap.add_argument("--sample", type=int, help="sub-sample size for median and IQR")
    ap.add_argument("--weights", type=float, nargs=4, metavar="w",
                    help="channel weights RGBA (1 1 1 1)")
    ap.add_argument("--fade", help="(clamp|repeat)/(abs|rel)/(f1,v1)/(f2,v2)[/...]")
    ap.add_argument("--threads", type=int, help="accepted for compatibility")
    ap.add_argument("--video-threads", type=int, help="accepted for compatibility")
    ap.add_argument("--shake-threads", type=int, help="accepted for compatibility")
    ap.add_argument("--shake", help="camera shake reduction: anchor-radius/search-radius")
    ap.add_argument("--shake-anchors", nargs="+", metavar="x/y", help="shake anchors x/y")
    ap.add_argument("-d", "--debug", action="store_true", help="print the parsed options")
    ap.add_argument("-w", "--wait", action="store_true", help="accepted for compatibility")
    return ap


def split_option_string(text):
    """Cli::from_str (src/cli.rs:238-258): the text split on '"'; outside quotes on spaces,
    a quoted part kept whole."""
    args = []
    for i, part in enumerate(text.split('"')):
        part = part.strip()
        if i % 2 == 0:
            args.extend(s for s in (x.strip() for x in part.split(" ")) if s)
        else:
            args.append(part)
    return args


def args_from_file(path):
    """The options of a .chrono file: its lines joined by spaces (src/main.rs:33-43)."""
    with open(path, encoding="utf-8") as f:
        content = f.read()
    return split_option_string(content.replace("\r\n", " ").replace("\n", " "))


def parse_range(s, name):
    """FrameRange::from_str (src/flist.rs:47-78): start/end/step, '.' for a default."""
    if s is None:
        return None
    parts = s.split("/")
    if len(parts) != 3:
        raise CliError("Option --%s expects 3 elements: start/end/step, %d were supplied"
                       % (name, len(parts)))
    vals = []
    for i, p in enumerate(parts):
        if p == ".":
            vals.append(None)
            continue
        try:
            vals.append(int(p))
        except ValueError:
            raise CliError("Can't parse element %d in option --%s (start/end/step), got '%s'"
                           % (i, name, p))
    return vals[0], vals[1], vals[2] if vals[2] is not None else 1


RANGE_OPTIONS = ("-f", "--frames", "--video-in", "--video-out")
RANGE_VALUE = re.compile(r"^-?(\d+|\.)/-?(\d+|\.)/(\d+|\.)$")


def _join_ranges(argv):
    """A range value may start with '-' (`--video-in -3/1/1`): joined to its option so that
    it is not read as an option itself."""
    out, i = [], 0
    while i < len(argv):
        a = argv[i]
        if a in RANGE_OPTIONS and i + 1 < len(argv) and RANGE_VALUE.match(argv[i + 1]):
            out.append(a + "=" + argv[i + 1])
            i += 2
        else:
            out.append(a)
            i += 1
    return out


def parse_args(argv):
    """Cli::parse (src/cli.rs:140-236): defaults, validation and the warnings for options
    that only --mode outlier uses. Returns (namespace, warnings)."""
    if len(argv) == 1 and not argv[0].startswith("-"):
        argv = args_from_file(argv[0])
    ns = build_parser().parse_args(_join_ranges(list(argv)))
    warnings = []
    if ns.mode is not None and ns.mode != "outlier":
        warnings = ["--" + k.replace("_", "-") for k in OUTLIER_ONLY
                    if getattr(ns, k) is not None]
    if (ns.shake is None) != (ns.shake_anchors is None):
        raise CliError("Provide both options or none: `--shake` and `--shake-anchors`")
    ns.mode = ns.mode or "outlier"
    ns.threshold = ns.threshold or "abs/0.05/0.2"
    ns.background = ns.background or "random"
    ns.outlier = ns.outlier or "extreme"
    if ns.quality is None:
        ns.quality = 95
    elif not 0 < ns.quality <= 100:
        raise CliError("Expected 0 < qualtiy <= 100. Got value %d" % ns.quality)
    ns.weights = list(ns.weights) if ns.weights else [1.0, 1.0, 1.0, 1.0]
    ns.frames = parse_range(ns.frames, "frames")
    ns.video_in = parse_range(ns.video_in, "video-in")
    ns.video_out = parse_range(ns.video_out, "video-out")
    if ns.shake is not None:
        try:
            r1, r2 = (int(v) for v in ns.shake.split("/"))
            anchors = [tuple(int(v) for v in a.split("/")) for a in ns.shake_anchors]
        except ValueError:
            raise CliError("--shake expects anchor-radius/search-radius and --shake-anchors x/y")
        if any(len(a) != 2 for a in anchors):
            raise CliError("--shake-anchors expects x/y pairs")
        ns.shake = (r1, r2)
        ns.shake_anchors = anchors
    # validated by the library's own parsers (Threshold, Fade), as the reference's FromStr
    api.Threshold.parse(ns.threshold)
    if ns.fade:
        api.Fade.parse(ns.fade)
    return ns, warnings


def list_files(pattern, frames):
    """FileLister::files_vec (src/flist.rs:94-120): the regular files matching the pattern in
    the glob crate's (sorted) order, then take(end).skip(start) and every step-th."""
    paths = [p for p in sorted(glob.glob(pattern)) if os.path.isfile(p)]
    if frames is None:
        return paths
    start, end, step = frames
    paths = paths[:end if end is not None else len(paths)][start or 0:]
    return [p for i, p in enumerate(paths) if i % step == 0]


def _decode(ctx, paths):
    if all(api._is_jpeg(p) for p in paths):
        return api.load_jpeg(paths, context=ctx)
    return api.load_png(paths, context=ctx)


def _numbered(path, frame, base_dir):
    """`{name}-{frame:05}.{ext}` in base_dir (src/main.rs:287-306; the blend mask's too is
    placed beside the composite output)."""
    stem, ext = os.path.splitext(os.path.basename(path))
    return os.path.join(base_dir, "%s-%05d%s" % (stem, frame, ext))


def _params(ns, n, seed):
    kw = dict(mode=ns.mode, threshold=ns.threshold, outlier=ns.outlier,
              background=ns.background, weights=ns.weights, fade=ns.fade, seed=seed)
    if ns.mode == "outlier" and ns.sample is not None and ns.sample < n:
        kw["sample"] = api.sample_indices(n, ns.sample, seed)
    return kw


def run(argv, out=sys.stdout):
    """main (src/main.rs:22-211): list files, optional shake analysis and crop, then one
    composite or one per video window, saved by extension."""
    ns, warnings = parse_args(argv)
    if warnings:
        print("WARNING! The following options are not used, as they are required only for "
              "`--mode outlier`:", file=out)
        for w in warnings:
            print(w, file=out)
        print(file=out)
    if ns.debug:
        print(vars(ns), file=out)
    files = list_files(ns.pattern, ns.frames)
    if not files:
        raise CliError("No files match the search pattern %r" % ns.pattern)
    ctx = api.default_context()
    frames = _decode(ctx, files)
    n, h, w, c = frames.shape
    crop = None
    if ns.shake is not None:
        offsets = api.ShakeAnalyzer(context=ctx).analyze(frames, ns.shake_anchors, ns.shake[0],
                                                          ns.shake[1])
        crops = api.Crop.create(offsets, w, h)
        if crops is not None:
            crop = (crops[:, :2], (int(crops[0, 2]), int(crops[0, 3])))
            print("Camera shake detected. Images will be corrected.", file=out)
        else:
            print("No camera shake detected. Images will not be corrected.", file=out)
    seed = 0x5EED
    blend = ns.mode == "outlier" and ns.output_blend is not None
    if ns.video_in is not None or ns.video_out is not None:
        vin = ns.video_in or (None, None, 1)
        vout = ns.video_out or (None, None, 1)
        base_dir = os.path.dirname(ns.output) or "."
        for frame, idx in api.video_windows(n, vin, vout):
            if not idx:
                continue
            sub_crop = None if crop is None else (crop[0][idx], crop[1])
            comp, bl = _composite(ctx, frames[idx], ns, sub_crop, idx[0], seed, blend)
            api.save_image(_numbered(ns.output, frame, base_dir), comp, quality=ns.quality,
                           context=ctx)
            if blend:
                api.save_image(_numbered(ns.output_blend, frame, base_dir), bl,
                               quality=ns.quality, context=ctx)
            print("Processing frame %d -> done" % frame, file=out)
    else:
        comp, bl = _composite(ctx, frames, ns, crop, 0, seed, blend)
        api.save_image(ns.output, comp, quality=ns.quality, context=ctx)
        if blend:
            api.save_image(ns.output_blend, bl, quality=ns.quality, context=ctx)
    return 0


def _composite(ctx, frames, ns, crop, offset, seed, blend):
    kw = _params(ns, frames.shape[0], seed)
    res = ctx.composite(np.ascontiguousarray(frames), blend=blend, crop=crop, frame_offset=offset,
                        **kw)
    return res[0], res[1]


def main(argv=None):
    try:
        return run(sys.argv[1:] if argv is None else argv)
    except (CliError, ValueError, api.ChronoError) as e:
        print("chrono-photo: %s" % e, file=sys.stderr)
        return 1
