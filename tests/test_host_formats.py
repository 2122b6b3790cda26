"""Host-side conversions to the reference's render-target formats: the GL
sRGB encoding of linear albedo into SRGB8 bytes round-trips every byte through
the GL decode, and is monotonic."""
import numpy as np

from dynamicradiancevolume_gb300 import pipeline


def _srgb_decode(b):
    """GL 4.5 section 8.24."""
    cs = np.asarray(b, np.float64) / 255.0
    return np.where(cs <= 0.04045, cs / 12.92, ((cs + 0.055) / 1.055) ** 2.4)


def test_srgb_encode_round_trips_every_byte():
    b = np.arange(256)
    assert np.array_equal(pipeline.srgb_encode(_srgb_decode(b)), b.astype(np.uint8))
    assert np.array_equal(pipeline.srgb_encode(_srgb_decode(b).astype(np.float32)), b.astype(np.uint8))


def test_srgb_encode_is_monotonic_and_clamped():
    lin = np.linspace(-0.5, 1.5, 20001)
    e = pipeline.srgb_encode(lin).astype(int)
    assert np.all(np.diff(e) >= 0)
    assert e[0] == 0 and e[-1] == 255
