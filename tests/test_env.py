"""The .env reader follows the reference's Environment rules (SDK/sutil/Environment.cpp)."""
import pytest

from pmdas_gb300 import env


def write(tmp_path, text):
    p = tmp_path / "scene.env"
    p.write_text(text)
    return str(p)


def test_defaults_match_registered_options():
    d = env.defaults()
    # optixMotionBlur.cpp:118-125
    assert d["mdas"] == 0 and d["samples"] == 1.0
    assert d["scaleFactor"] == 1.0 and d["alpha"] == 0.25
    assert d["bitsPerDim"] == 0 and d["extraImgBits"] == 8 and d["candidatesNum"] == 4
    assert d["width"] == 1024 and d["height"] == 768 and d["fovy"] == 45.0
    assert d["sceneKind"] == -1


def test_sampler_and_mdas_blocks(tmp_path):
    p = write(tmp_path, """
# a comment line
Sampler {
    mdas true
    samples 8      # trailing comment
}
Mdas {
    scaleFactor 0.0625
    alpha 0.015625
    bitsPerDim 1
    extraImgBits 7
    candidatesNum 6
}
Film { width 640 height 480 filename out.exr }
Camera { position 0 0 1 direction 0 0 -1 fovy 30 focalDistance 4 lensRadius 0.1 }
Light { color 1 1 1| point 0 1 2 color 0.5 0.5 0.5 }
Scene { kind dof seed 42 count 256 }
""")
    d = env.read_env(p)
    assert d["mdas"] == 1 and d["samples"] == 8.0
    assert d["scaleFactor"] == 0.0625 and d["alpha"] == 0.015625
    assert (d["bitsPerDim"], d["extraImgBits"], d["candidatesNum"]) == (1, 7, 6)
    assert (d["width"], d["height"], d["filmFilename"]) == (640, 480, "out.exr")
    assert d["fovy"] == 30.0 and d["focalDistance"] == 4.0 and abs(d["lensRadius"] - 0.1) < 1e-7
    assert (d["sceneKind"], d["sceneSeed"], d["sceneCount"]) == (1, 42, 256)


def test_float_values_keep_six_decimals(tmp_path):
    # values are stored as std::to_string(float): 6 decimals (Environment.cpp:17-20)
    d = env.read_env(write(tmp_path, "Mdas { alpha 0.0000004 scaleFactor 0.1234567 }"))
    assert d["alpha"] == 0.0
    import numpy as np
    assert d["scaleFactor"] == np.float32(0.123457)


def test_first_occurrence_wins(tmp_path):
    d = env.read_env(write(tmp_path, "Mdas { alpha 0.5 }\nMdas { alpha 0.125 }"))
    assert d["alpha"] == 0.5


@pytest.mark.parametrize("text,msg", [
    ("Mdas { beta 1 }", "Unknown option 'Mdas.beta'"),
    ("Sampler { mdas maybe }", "Mismatch"),
    ("Mdas { alpha", "Mismatch"),  # a value must follow on the same line
    ("Camera { position 1 2", "Mismatch"),
    ("}", "Unpaired }"),
    ("Scene { kind teapot }", "Unknown Scene.kind"),
])
def test_errors(tmp_path, text, msg):
    with pytest.raises(ValueError) as e:
        env.read_env(write(tmp_path, text))
    assert msg in str(e.value)


def test_missing_file():
    with pytest.raises(ValueError) as e:
        env.read_env("/nonexistent/x.env")
    assert "Cannot open" in str(e.value)


def test_bool_spellings(tmp_path):
    for word, want in (("yes", 1), ("ON", 1), ("1", 1), ("off", 0), ("FALSE", 0), ("no", 0)):
        assert env.read_env(write(tmp_path, f"Sampler {{ mdas {word} }}"))["mdas"] == want
