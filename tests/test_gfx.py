"""Headless snapshots (pyfds/gfx.py:14-404): the recorder's frames against the
oracle's state at the frame steps (GPU), and the constructor's checks (CPU)."""
import numpy as np
import pytest

from oracle import fds_oracle as O
from oracle import scenarios as S
from helpers import build_field


def _field():
    spec = S.random_scenario(5, "Acoustic2D", 24, 10, steps=20, mu=False)
    spec["nt"] = 20
    return spec, build_field(spec, exact=True)


def test_animator_checks():
    import pyfds_gb300 as fds
    _, f = _field()
    with pytest.raises(KeyError):
        fds.Animator2D(f, observed_component="temperature")
    with pytest.raises(ValueError):
        fds.Animator2D(f, scale=[1, 2, 3])
    a = fds.Animator2D(f, observed_component="velocity_x", scale=2)
    assert a.scale == (-2, 2) and a.observed_component == "velocity_x"
    assert fds.Animator2D(f).observed_component == "pressure"
    m = a.field_as_matrix(np.arange(240.0))
    assert m.shape == (10, 24) and m[1, 0] == 24.0
    with pytest.raises(NotImplementedError):
        a.show_setup()


@pytest.mark.gpu
def test_frames_match_oracle(gpu, tmp_path):
    import pyfds_gb300 as fds
    spec, f = _field()
    a = fds.Animator2D(f, observed_component="velocity_y", steps_per_frame=6, save_video=True,
                       video_file_name=str(tmp_path / "frames.mp4"))
    frames = a.start_simulation()
    assert frames.shape == (3, 10, 24) and f.step == 18
    state = None
    for k in range(3):
        state, _ = O.simulate(spec, 6, state=state, step0=6 * k)
        assert np.array_equal(frames[k].cpu().numpy().reshape(-1), state["velocity_y"]), k
    assert np.allclose(a.frame_times, [f.t.vector[5], f.t.vector[11], f.t.vector[17]])
    saved = np.load(tmp_path / "frames.npz")
    assert np.array_equal(saved["frames"], frames.cpu().numpy())
