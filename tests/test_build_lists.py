"""The specialised kernel variants are listed twice, in cp_internal.h (declarations and the
launch dispatch) and in build.py (what gets compiled): the two lists must agree."""
import os
import re

from chrono_photo_gb300 import build

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    "chrono_photo_gb300", "csrc")


def _x_list(name):
    """The (channels, kind, group, background) entries of the X-macro list `name`."""
    text = open(os.path.join(CSRC, "cp_internal.h")).read()
    start = text.index("#define %s(X)" % name)
    body = text[start:text.index("\n#define", start + 1)]
    return sorted(tuple(int(v) for v in t) for t in
                  re.findall(r"X\((\d+), (\d+), (\d+), (\d+)\)", body))


def test_single_stack_variants_match_build():
    assert _x_list("CP_VARIANTS") == sorted(build.KERNEL_VARIANTS)


def test_batch_variants_match_build():
    assert _x_list("CP_BATCH_VARIANTS") == sorted(build.BATCH_VARIANTS)


def test_pixel_thread_variants_match_build():
    text = open(os.path.join(CSRC, "cp_internal.h")).read()
    start = text.index("#define CP_PX_VARIANTS(X)")
    body = text[start:text.index("\n#define", start + 1)]
    listed = sorted(tuple(int(v) for v in t)
                    for t in re.findall(r"X\((\d+), (\d+), (\d+)\)", body))
    assert listed == sorted(build.PX_VARIANTS)
    assert len(listed) == 12


def test_every_rgb_outlier_setting_has_a_variant():
    """Every (distance kind, outlier group, background) an RGB stack can map to is compiled."""
    have = set(build.KERNEL_VARIANTS)
    for k in (1, 2):
        for g in (1, 2, 3):
            for b in (0, 1):
                assert (3, k, g, b) in have
    assert (3, 3, 0, 0) in have
    for ch in (1, 4):
        for k in (1, 2, 3):
            assert (ch, k, 0, 0) in have
