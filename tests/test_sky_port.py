"""The atmosphere background of the C restatement (oracle/port) against the reference's own
code: the scattering table of AtmosphereApp::precomputeTable against the table the
reference ships and loads (resources/common/scattering-precomputed.exr), and
MaterialSky::eval against the reference's evaluations with that table
(tests/golden/sky.npz, made by tests/golden/make_golden.py --sky)."""
import numpy as np

from conftest import load_golden


def test_half_rounding_matches_ieee(port_lib):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(0, 1, 2000), np.exp(rng.uniform(-30, 11, 2000)) * rng.choice([-1, 1], 2000),
                        [0.0, -0.0, 65504.0, 65519.0, 6e-8, 2.9802322e-08, 1e-10]]).astype(np.float32)
    np.testing.assert_array_equal(port_lib.port_round_half(x).view(np.uint32),
                                  x.astype(np.float16).astype(np.float32).view(np.uint32))


def test_port_table_is_the_shipped_table(port_lib):
    """512 x 512, 256 samples, stored in half precision: equal to the shipped table except
    where expf's last-bit rounding lands on the other side of a half-precision tie."""
    g = load_golden("sky.npz")
    t = port_lib.port_sky_table(512, 256)
    assert tuple(g["table_shape"]) == t.shape
    sub = t[::8, ::8, :3]
    assert (sub == g["table_sub"]).mean() > 0.999
    np.testing.assert_allclose(sub, g["table_sub"], rtol=2 ** -10, atol=2 ** -24)
    np.testing.assert_allclose(t[..., :3].astype(np.float64).sum(axis=1), g["table_row_sums"], rtol=1e-5, atol=1e-6)


def test_port_sky_matches_reference(port_lib):
    """MaterialSky::eval: the restatement with its own table against the reference with the
    shipped one (bit-identical evaluations where the two tables agree)."""
    g = load_golden("sky.npz")
    t = port_lib.port_sky_table(512, 256)
    out = port_lib.port_sky_eval(t, g["cases"])
    ref = g["eval_out"]
    assert (out == ref).all(axis=1).mean() > 0.99
    np.testing.assert_allclose(out, ref, rtol=2e-3, atol=1e-6)
    # the sun disc: rays within the disc see sun radiance of order 1e3
    assert ref[:750].max() > 1e3
