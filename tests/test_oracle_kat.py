"""The oracle against the golden known answers (CPU only).

Pins both CPU restatements (oracle/chrono_oracle.cpp and oracle/pyref.py) to the
reference's own quartiles_test (src/chrono.rs:598-604) and to hand-derived answers for each
quirk of the reference's arithmetic (tests/golden/kat.json)."""
import numpy as np
import pytest

from oracle import oracle, pyref
from tests import cases

KAT = cases.kat()


@pytest.mark.parametrize("case", KAT["quartiles"], ids=lambda c: c["name"])
def test_quartiles(case):
    assert oracle.quartiles(case["sorted"]) == tuple(case["expect"])
    d = case["sorted"]
    got = (pyref.quantile(d, 0.25), pyref.median(d), pyref.quantile(d, 0.75))
    assert tuple(float(x) for x in got) == tuple(case["expect"])


def test_quartiles_rejects_short():
    with pytest.raises(ValueError):
        oracle.quartiles([1, 2])


def _pixel_params(case):
    return cases.params(mode="outlier", threshold=case["threshold"], outlier=case["outlier"],
                        background=case["background"], weights=case["weights"],
                        fade=case.get("fade"))


@pytest.mark.parametrize("case", KAT["pixels"], ids=lambda c: c["name"])
def test_pixel_kat_oracle(case):
    st = cases.pixel_stack(case["samples"])
    out, blend, warn, dbg = oracle.composite(st, _pixel_params(case), debug=True)
    assert out.reshape(-1).tolist() == case["expect_pixel"]
    c = len(case["expect_pixel"])
    assert blend.reshape(-1)[: min(c, 3)].tolist() == [case["expect_mask"]] * min(c, 3)
    if "expect_mask_alpha" in case:
        assert blend.reshape(-1)[3] == case["expect_mask_alpha"]
    bits = int(dbg["outlier_bits"].reshape(-1)[0])
    assert [i for i in range(len(case["samples"])) if bits >> i & 1] == case["expect_outliers"]
    if "expect_background" in case:
        assert int(dbg["background"].reshape(-1)[0]) == case["expect_background"]


@pytest.mark.parametrize("case", KAT["pixels"], ids=lambda c: c["name"])
def test_pixel_kat_pyref(case):
    from chrono_photo_gb300.api import Fade, Threshold
    thr = Threshold.parse(case["threshold"])
    t = pyref.Threshold(thr.absolute, thr.min, thr.max)
    fd = Fade.parse(case["fade"]) if case.get("fade") else Fade.none()
    fade = pyref.fade_table(fd.repeat, fd.absolute, fd.points)
    pix, mask, warn, det = pyref.calc_pixel([tuple(s) for s in case["samples"]], t,
                                            case["weights"], case["background"],
                                            case["outlier"], fade, 0)
    assert list(pix) == case["expect_pixel"]
    assert mask == case["expect_mask"]
    assert det["outliers"] == case["expect_outliers"]


@pytest.mark.parametrize("case", KAT["simple"], ids=lambda c: c["name"])
def test_simple_kat(case):
    st = cases.pixel_stack(case["samples"])
    p = cases.params(mode="darker" if case["darker"] else "lighter", weights=case["weights"],
                     fade=case.get("fade"))
    out, _, _ = oracle.composite(st, p)
    assert out.reshape(-1).tolist() == case["expect_pixel"]
    from chrono_photo_gb300.api import Fade
    fd = Fade.parse(case["fade"]) if case.get("fade") else Fade.none()
    fade = pyref.fade_table(fd.repeat, fd.absolute, fd.points)
    assert list(pyref.simple_pixel([tuple(s) for s in case["samples"]], case["weights"],
                                   case["darker"], fade, 0)) == case["expect_pixel"]


@pytest.mark.parametrize("case", KAT["crop"])
def test_crop_kat(case):
    got = oracle.crop_create(case["offsets"], case["width"], case["height"])
    if case["expect"] is None:
        assert got is None
    else:
        assert got.tolist() == case["expect"]


@pytest.mark.parametrize("case", KAT["windows"])
def test_windows_kat(case):
    got = oracle.video_windows(case["image_count"], tuple(case["video_in"]),
                               tuple(case["video_out"]))
    assert [[f, idx] for f, idx in got] == case["expect"]


def test_shake_uniform_first_minimum():
    frames = np.full((3, 40, 40, 3), 77, np.uint8)
    offs = oracle.shake(frames, [(20, 20)], r=3, s=4)
    assert offs.tolist() == [[0, 0], [-4, -4], [-4, -4]]


def test_shake_exact_shift():
    rng = np.random.default_rng(7)
    big = rng.integers(0, 256, size=(80, 80, 3), dtype=np.uint8)
    f0 = big[10:70, 10:70]
    f1 = big[10 - 2:70 - 2, 10 + 3:70 + 3]  # content moves by (-3, +2)
    offs = oracle.shake(np.stack([f0, f1]), [(30, 30)], r=5, s=6)
    assert offs.tolist() == [[0, 0], [-3, 2]]


def test_shake_wrapping_sum():
    """Sums above 2^31 wrap in i32 (release profile): the wrapped value is what min_by_key
    compares. Recompute one offset's sum with Python integers modulo 2^32."""
    r, s = 53, 1
    size = 2 * r + 1
    h = w = size + 2 * s + 2
    f0 = np.zeros((h, w, 3), np.uint8)
    f1 = np.full((h, w, 3), 255, np.uint8)
    f1[0, 0] = 0
    c = (w // 2, h // 2)
    offs, dd = oracle.shake(np.stack([f0, f1]), [c], r=r, s=s, diffs=True)
    full = size * size * 3 * 255 * 255
    wrapped = (full + 2 ** 31) % 2 ** 32 - 2 ** 31
    assert full > 2 ** 31 and dd[0, 1, 1] == wrapped
    k = int(np.argmin(dd[0].reshape(-1)))
    assert offs[1].tolist() == [k % 3 - s, k // 3 - s]
