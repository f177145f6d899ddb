"""The command line end to end on JPEG frames (needs a GB300): each output file holds what
the library's API gives for the same decoded frames (PNG outputs compared sample for sample,
JPEG outputs byte for byte through the same encoder)."""
import os

import numpy as np
import pytest

import chrono_photo_gb300 as cg
from chrono_photo_gb300 import cli
from tests import cases

pytestmark = pytest.mark.gpu


@pytest.fixture
def jpeg_frames(tmp_path):
    rng = np.random.default_rng(31)
    frames = cases.random_stack(rng, 12, 48, 64, 3, n_spots=3)
    d = tmp_path / "frames"
    d.mkdir()
    for i, f in enumerate(frames):
        cg.save_jpeg(d / ("image-%05d.jpg" % i), f, quality=95)
    return str(d / "*.jpg"), sorted(str(p) for p in d.iterdir())


def test_outlier_with_blend(ctx, tmp_path, jpeg_frames):
    pattern, paths = jpeg_frames
    out, blend = str(tmp_path / "out.png"), str(tmp_path / "masks" / "blend.png")
    assert cli.run(["-p", pattern, "-o", out, "--output-blend", blend, "-b", "first",
                    "-l", "average", "-t", "abs/0.05/0.2"]) == 0
    frames = cg.load_jpeg(paths, context=ctx)
    ref = ctx.composite(frames, mode="outlier", threshold="abs/0.05/0.2", background="first",
                        outlier="average")
    assert np.array_equal(cg.load_png([out])[0], ref[0])
    assert np.array_equal(cg.load_png([blend])[0], ref[1])


def test_darker_to_jpeg_with_frame_range(ctx, tmp_path, jpeg_frames):
    pattern, paths = jpeg_frames
    out = str(tmp_path / "dark.jpg")
    assert cli.run(["-p", pattern, "-o", out, "-m", "darker", "-f", "1/10/2", "-q", "90"]) == 0
    sel = paths[1:10][::2]
    frames = cg.load_jpeg(sel, context=ctx)
    ref = ctx.composite(frames, mode="darker", blend=False)[0]
    assert open(out, "rb").read() == cg.encode_jpeg(ref, quality=90)


def test_video_windows_and_options_file(ctx, tmp_path, jpeg_frames):
    pattern, paths = jpeg_frames
    out = tmp_path / "video" / "frame.png"
    out.parent.mkdir()
    opts = tmp_path / "video.chrono"
    opts.write_text('--pattern "%s"\n--output "%s"\n--video-in -3/1/1\n--background first\n'
                    '--outlier extreme\n' % (pattern, out))
    assert cli.run([str(opts)]) == 0
    frames = cg.load_jpeg(paths, context=ctx)
    wins = cg.video_windows(len(paths), (-3, 1, 1), (None, None, 1))
    assert any(idx for _, idx in wins)
    for frame, idx in wins:
        path = out.parent / ("frame-%05d.png" % frame)
        if not idx:  # an empty window writes no frame (the reference prints "Skipping")
            assert not path.exists()
            continue
        assert path.exists(), path
        ref = ctx.composite(np.ascontiguousarray(frames[idx]), mode="outlier",
                            threshold="abs/0.05/0.2", background="first", outlier="extreme",
                            frame_offset=idx[0])[0]
        assert np.array_equal(cg.load_png([str(path)])[0], ref)


def test_errors_exit_with_status(tmp_path, capsys):
    assert cli.main(["-p", str(tmp_path / "none*.jpg"), "-o", str(tmp_path / "o.png")]) == 1
    assert "No files match" in capsys.readouterr().err
    assert cli.main(["-p", "x", "-o", "o.png", "-q", "0"]) == 1
