"""The command line (chrono_photo_gb300/cli.py) on the CPU: the reference's defaults and
option parsing (src/cli.rs), options files (src/main.rs:33-43), the file lister's frame
range (src/flist.rs) and the numbered outputs of chrono-video (src/main.rs:287-306)."""
import os

import pytest

from chrono_photo_gb300 import cli


def test_defaults():
    ns, warnings = cli.parse_args(["-p", "frames/*.jpg", "-o", "out.jpg"])
    assert (ns.mode, ns.threshold, ns.background, ns.outlier, ns.quality) == \
        ("outlier", "abs/0.05/0.2", "random", "extreme", 95)
    assert ns.weights == [1.0, 1.0, 1.0, 1.0] and ns.fade is None and ns.sample is None
    assert ns.frames is None and ns.video_in is None and ns.shake is None and warnings == []


def test_reference_args_from_string():
    """The reference's own CLI test (src/cli.rs:345-352): a quoted pattern and four weights."""
    s = ('--pattern "test_data/generated/*.jpg" --output test_data/temp --weights 0 1 1 0')
    ns, _ = cli.parse_args(cli.split_option_string(s))
    assert ns.pattern == "test_data/generated/*.jpg" and ns.weights == [0, 1, 1, 0]


def test_options_file(tmp_path):
    f = tmp_path / "opts.chrono"
    f.write_text('--pattern "my frames/*.jpg"\r\n--output out.png\n--mode darker\n'
                 '--frames 2/./3\n--fade clamp/abs/0,0/8,1\n')
    ns, _ = cli.parse_args([str(f)])
    assert ns.pattern == "my frames/*.jpg" and ns.mode == "darker"
    assert ns.frames == (2, None, 3) and ns.fade == "clamp/abs/0,0/8,1"


def test_short_options_and_shake():
    ns, _ = cli.parse_args(["-p", "a*", "-o", "o.png", "-m", "outlier", "-t", "rel/2/4",
                            "-b", "first", "-l", "forward", "-q", "80", "--sample", "10",
                            "--shake", "32/20", "--shake-anchors", "100/50", "200/80",
                            "--video-in", "-3/1/1", "--video-out", "././2"])
    assert (ns.threshold, ns.background, ns.outlier, ns.quality, ns.sample) == \
        ("rel/2/4", "first", "forward", 80, 10)
    assert ns.shake == (32, 20) and ns.shake_anchors == [(100, 50), (200, 80)]
    assert ns.video_in == (-3, 1, 1) and ns.video_out == (None, None, 2)


@pytest.mark.parametrize("argv,what", [
    (["-p", "a", "-o", "o", "-q", "0"], "qualtiy"),
    (["-p", "a", "-o", "o", "-q", "101"], "qualtiy"),
    (["-p", "a", "-o", "o", "--shake", "3/4"], "--shake-anchors"),
    (["-p", "a", "-o", "o", "--frames", "1/2"], "3 elements"),
    (["-p", "a", "-o", "o", "--frames", "1/x/2"], "Can't parse"),
])
def test_errors(argv, what):
    with pytest.raises(cli.CliError) as e:
        cli.parse_args(argv)
    assert what in str(e.value)


def test_bad_threshold_and_fade():
    with pytest.raises(ValueError):
        cli.parse_args(["-p", "a", "-o", "o", "-t", "sqrt/1"])
    with pytest.raises(ValueError):
        cli.parse_args(["-p", "a", "-o", "o", "--fade", "clamp/abs/0"])


def test_outlier_only_options_warn():
    _, warnings = cli.parse_args(["-p", "a", "-o", "o", "-m", "lighter", "-t", "abs/0.1",
                                  "--output-blend", "b.png", "--sample", "4"])
    assert set(warnings) == {"--threshold", "--output-blend", "--sample"}


def test_file_lister_frame_range(tmp_path):
    for i in range(10):
        (tmp_path / ("img-%02d.jpg" % (9 - i))).write_bytes(b"x")
    (tmp_path / "dir.jpg").mkdir()  # not a regular file
    pat = str(tmp_path / "*.jpg")
    names = [os.path.basename(p) for p in cli.list_files(pat, None)]
    assert names == ["img-%02d.jpg" % i for i in range(10)]
    got = [os.path.basename(p) for p in cli.list_files(pat, (2, 9, 3))]
    assert got == ["img-02.jpg", "img-05.jpg", "img-08.jpg"]
    got = [os.path.basename(p) for p in cli.list_files(pat, (None, 4, 1))]
    assert got == ["img-00.jpg", "img-01.jpg", "img-02.jpg", "img-03.jpg"]


def test_numbered_outputs():
    assert cli._numbered("out/video.jpg", 7, "out") == os.path.join("out", "video-00007.jpg")
    assert cli._numbered("masks/b.png", 12, "out") == os.path.join("out", "b-00012.png")
