"""The .sph-config reader (sim/config-parser.go grammar, fields and messages)."""
import ctypes as C

import numpy as np
import pytest

from sphugo_gb300 import sim as S

FULL = """// a complete configuration
// comments start with two slashes

[[Simulation]]
[Config]
NSteps              250
Gamma               1.4
ParticleMass        0.5
Acceleration        0       -0.25
DeltaTHalf          0.002
Kernel              Wendtland

[[Start]]

[UniformRect]
NParticles          120
UpperLeft           0.1     0.2
LowerRight          0.3     0.4

[UniformRect]
LowerRight          0.9     0.8
NParticles          120
UpperLeft           0.5     0.6

[[Boundaries]]
[Periodic]
Horizontal          0.0       1.0
Vertical            -2      2
[Reflection]
Down                0.95
Left   0.05

[[Sources]]
[Point]
Pos               0.5     0.5
Rate              20

[[Simulation]]
[Viewport]
UpperLeft           0       0
LowerRight          2       1
"""


def load(tmp_path, text, name="c.sph-config"):
    p = tmp_path / name
    p.write_text(text)
    cfg, err = S.MakeConfigFromFile(str(p))
    return cfg, err, str(p)


def test_full_config(sphlib, tmp_path):
    cfg, err, _ = load(tmp_path, FULL)
    assert err is None
    assert cfg.NSteps == 250 and cfg.Gamma == 1.4 and cfg.ParticleMass == 0.5
    assert (cfg.Acceleration.X, cfg.Acceleration.Y) == (0.0, -0.25)
    assert cfg.DeltaTHalf == 0.002 and cfg.Kernel == "Wendtland"
    assert len(cfg.Start) == 2 and cfg.Start[1].NParticles == 120
    assert (cfg.Start[1].UpperLeft.X, cfg.Start[1].LowerRight.Y) == (0.5, 0.8)
    assert cfg.HorPeriodicity == (0.0, 1.0) and cfg.VertPeriodicity == (-2.0, 2.0)
    assert cfg.Reflections.D == 0.95 and cfg.Reflections.L == 0.05 and cfg.Reflections.R == S.DBL_MAX
    assert len(cfg.Sources) == 1 and cfg.Sources[0].rate == 20.0 and cfg.Sources[0].origin.X == 0.5
    assert cfg.Viewport == ((0.0, 0.0), (2.0, 1.0))


def test_defaults_of_makeconfig(sphlib):
    c = S.MakeConfig()
    assert (c.Gamma, c.NSteps, c.DeltaTHalf, c.ParticleMass, c.Kernel) == (1.66666, 10000, 0.001, 1.0, "Monahan")
    assert c.HorPeriodicity == (-S.DBL_MAX, S.DBL_MAX)


def test_added_keys(sphlib, tmp_path):
    text = ("[[Simulation]]\n[Config]\nNeighbourCount 64\nViscosityAlpha 1\nViscosityBeta 2.0\n"
            "ViscosityEtaSq 0.005\nPrecision Mixed\nGridLevel 9\n")
    cfg, err, _ = load(tmp_path, text)
    assert err is None
    assert (cfg.NeighbourCount, cfg.ViscosityAlpha, cfg.ViscosityBeta, cfg.ViscosityEtaSq) == (64, 1.0, 2.0, 0.005)
    assert cfg.Precision == "Mixed" and cfg.GridLevel == 9


@pytest.mark.parametrize("text,msg", [
    ("[[Foo]]\n", "1:3: ConfigMakeError: `Foo` is not a valid title\n"),
    ("[[Simulation]]\n[Bar]\n",
     "2:2: ConfigMakeError: `Bar` is not a valid subtitle under title: `Simulation`. "
     "It's valid subtitles are: [Config Viewport]\n"),
    ("[[Simulation]]\n[Config]\nKernel Gaussian\n", "3:7: ConfigMakeError: Kernel `Gaussian` is not implemented\n"),
    ("[[Simulation]]\n[Config]\nNSteps 1.5\n", "3:7: ConfigMakeError: expected an integer but got something else\n"),
    ("[[Simulation]]\n[Config]\nWhat 1\n",
     "3:5: ConfigMakeError: `What` is not a valid parameter in `[[Simulation]]` - `[Config]`\n"),
    ("[Config]\n", "1:2: ConfigMakeError: Expected a [[Title]] but got `subtitle`\n"),
    ("[[Simulation]]\nGamma 2\n", "2:6: ConfigMakeError: Expected a [Subtitle] but got `integer`\n"),
    ("/ x\n", "1:2: ConfigParseError: Expected `/`, but we got this: ` `\n"),
    ("[[Simulation]]\n[Config]\nAcceleration 1 2 3\n",
     "3:19: ConfigParseError: Cannot parse a Vector with more than 2 dimensions\n"),
    ("[[Simulation]]\n[Config]\nGamma 1x\n", "3:8: ConfigParseError: In number literal expected a `.` or a digit\n"),
])
def test_error_messages(sphlib, tmp_path, text, msg):
    cfg, err, path = load(tmp_path, text)
    assert err is not None
    assert str(err) == f"{path}:{msg}"
    assert cfg == S.MakeConfig()  # a failed load yields the defaults


def test_two_dots_form_a_vector(sphlib, tmp_path):
    # "1.5.3" tokenises as the two numbers 1.5 and .3, so Gamma rejects a vec2
    cfg, err, path = load(tmp_path, "[[Simulation]]\n[Config]\nGamma 1.5.3\n")
    assert "expected an integer or float but got something else" in str(err)


def test_uniform_rect_needs_three_params(sphlib, tmp_path):
    text = "[[Start]]\n[UniformRect]\nNParticles 10\nUpperLeft 0 0\n[[Boundaries]]\n[Reflection]\nDown 1\n"
    cfg, err, _ = load(tmp_path, text)
    # the title that follows is taken as the third parameter; its empty name
    # matches the reference's pre-filled `got` list
    assert "The parameter name `` in [`UniformRect`] is already set!" in str(err)
    text = "[[Start]]\n[UniformRect]\nNParticles 10\nNParticles 5\nUpperLeft 0 0\n[[Boundaries]]\n"
    cfg, err, _ = load(tmp_path, text)
    assert "The parameter name `NParticles` in [`UniformRect`] is already set!" in str(err)


def test_viewport_type_errors_are_ignored(sphlib, tmp_path):
    cfg, err, _ = load(tmp_path, "[[Simulation]]\n[Viewport]\nUpperLeft 3\nLowerRight 4 5\n")
    assert err is None and cfg.Viewport == ((0.0, 0.0), (4.0, 5.0))


def test_value_at_end_of_file_without_newline(sphlib, tmp_path):
    cfg, err, _ = load(tmp_path, "[[Simulation]]\n[Config]\nNSteps 7")
    assert err is None and cfg.NSteps == 7


def test_missing_file_is_an_error(sphlib, tmp_path):
    cfg, err = S.MakeConfigFromFile(str(tmp_path / "nope.sph-config"))
    assert err is not None and "cannot read" in str(err)


def test_spawners_reseed_per_spawner(sphlib, tmp_path):
    cfg, err, _ = load(tmp_path, FULL)
    x, y, vx, vy, u = S.spawn_start(cfg)
    assert len(x) == 240 and np.all(u == 0.01) and np.all(vx == 0)
    a, b = slice(0, 120), slice(120, 240)
    # same stream for both spawners: identical relative positions
    rx0 = (x[a] - 0.1) / 0.2
    rx1 = (x[b] - 0.5) / 0.4
    assert np.allclose(rx0, rx1, rtol=0, atol=1e-12)
    assert 0.1 <= x[a].min() and x[a].max() < 0.3 and 0.6 <= y[b].min() and y[b].max() < 0.8


def test_point_source_rate(sphlib):
    from sphugo_gb300 import _lib as L
    src = L.SphPointSource()
    src.origin[:] = (0.5, 0.5)
    src.rate = 10.0
    lib = L.load()
    x, y = np.empty(8), np.empty(8)
    n = lib.sph_point_source_spawn(C.byref(src), 0.35, 1, L.dptr(x), L.dptr(y), None, None, None, None)
    assert n == 3 and src.last_spawned == pytest.approx(0.3)
    assert np.all(np.abs(x[:3] - 0.5) <= 0.01)
    assert lib.sph_point_source_spawn(C.byref(src), 0.45, 2, None, None, None, None, None, None) == 1
