"""The text dump and the command-line driver's flags, on CPU: the library's
threaded writer against np.savetxt(fh, a.reshape(-1, last_dim),
delimiter=",") byte for byte (pyminiweather/__main__.py:220-233), and the
parser against the reference driver's flags and defaults
(pyminiweather/__main__.py:28-156)."""
import io

import numpy as np
import pytest

from pyminiweather_gb300.__main__ import get_params_from_args, get_parser
from pyminiweather_gb300.post.output import savetxt, svars_filename


def _np_bytes(arrays):
    fh = io.BytesIO()
    for a in arrays:
        a = np.asarray(a, dtype=np.float64)
        np.savetxt(fh, a.reshape(-1, a.shape[-1]), delimiter=",")
    return fh.getvalue()


def _special_values():
    rng = np.random.default_rng(7)
    v = np.concatenate([
        [0.0, -0.0, 1.0, -1.0, 1 / 3, -2 / 3, 0.1, 1e-300, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
         -1.7976931348623157e308, 1e22, 9.999999999999999e22, 123456789012345678.0, np.nan, -np.nan, np.inf, -np.inf,
         0.5e-5, 299.99999999999994, 1e100, 1e-100],
        rng.standard_normal(200) * 10.0 ** rng.integers(-30, 30, 200),
        rng.uniform(-1, 1, 120)])
    return v


@pytest.mark.parametrize("shape", [(343,), (7, 49), (3, 7, 7 * 7 // 7), (1, 1)])
def test_savetxt_matches_numpy_bytes(tmp_path, shape):
    v = _special_values()
    n = int(np.prod(shape))
    a = np.resize(v, n).reshape(shape)
    path = tmp_path / "out.txt"
    savetxt(str(path), a)
    assert path.read_bytes() == _np_bytes([a])


def test_savetxt_append_and_threads(tmp_path):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((4, 37, 53)) * 1e3
    b = rng.standard_normal((4, 37, 53))
    p1, p2 = tmp_path / "a.txt", tmp_path / "b.txt"
    savetxt(str(p1), a, threads=1)
    savetxt(str(p1), b, append=True, threads=1)
    savetxt(str(p2), a, threads=7)
    savetxt(str(p2), b, append=True, threads=7)
    ref = _np_bytes([a, b])
    assert p1.read_bytes() == ref and p2.read_bytes() == ref


def test_svars_filename():
    assert svars_filename("PyMiniWeatherData.txt") == "PyMiniWeatherData_svars.txt"
    with pytest.raises(ValueError):  # the reference splits on a single '.'
        svars_filename("a.b.txt")


def test_cli_flags_and_defaults_match_the_reference():
    p = get_parser()
    args = p.parse_args([])
    ref_defaults = dict(nx=200, nz=100, xlen=2e4, zlen=1e4, nsteps=10, dt=None, nwarmups=0, ic_type="thermal", hs=2,
                        s=4, max_speed=500.0, cfl=1.0, verbose=False, output_freq=-1,
                        app_filename="PyMiniWeatherData.txt", app_log_file=None)
    for k, v in ref_defaults.items():
        assert getattr(args, k) == v, k
    a = p.parse_args(["--nx", "64", "--nz", "32", "--ic-type", "collision", "--max-speed", "450", "--cfl", "1.5",
                      "--output-freq", "5", "--app-filename", "x.txt", "--nwarmups", "2", "--dt", "0.5", "--verbose"])
    params = get_params_from_args(a)
    assert (params["nx"], params["nz"], params["ic_type"], params["max_speed"], params["cfl"], params["output_freq"],
            params["app_filename"], params["nwarmups"], params["dt"], params["verbose"]) == (
        64, 32, "collision", 450.0, 1.5, 5, "x.txt", 2, 0.5, True)
    with pytest.raises(SystemExit):
        p.parse_args(["--hs", "3"])  # fixed at 2, as in the reference
