"""Procedural keyframe generator (input infrastructure)."""
import numpy as np

from imagebasedspatiotemporalinterpolation_gb300.scene import SplitMix64, Sequence


def test_splitmix64_known_values():
    # SplitMix64 reference outputs for seed 1234567 (Steele, Lea, Flood 2014 algorithm)
    r = SplitMix64(1234567)
    assert [r.next_u64() for _ in range(3)] == [6457827717110365317, 3203168211198807973, 9817491932198370423]


def test_sequence_buffers(built):
    seq = Sequence(96, 54, 3, seed=9, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0)
    fr = seq.frame(1)
    assert len(fr.views()) == 6 and fr.aux_priority == [3, 3]
    for v in fr.views():
        assert v.color.shape == (54, 96, 4) and v.color.dtype == np.uint8 and (v.color[..., 3] == 255).all()
        assert v.z.dtype == np.float32 and (v.z >= -1).all() and (v.z <= 1).all()
        assert v.motion.dtype == np.float16 and v.motion.shape == (54, 96, 3)
        m4 = v.motion_f32x4()
        assert m4.dtype == np.float32 and (m4[..., 3] == 0).all()
        assert np.array_equal(m4[..., :3].astype(np.float16), v.motion)
        assert v.shadow_info is not None and v.shadow_a is not None and v.shadow_b is not None
    # the same seed reproduces the same buffers
    again = Sequence(96, 54, 3, seed=9, aux_offsets=(-0.3, 0.3), shadows=True, max_speed=3.0).frame(1)
    assert np.array_equal(again.fwd.z, fr.fwd.z) and np.array_equal(again.bwd.color, fr.bwd.color)


def test_client_camera_between_keyframes(built):
    seq = Sequence(64, 36, 3, seed=2)
    c0, c4 = seq.client(0, 0), seq.client(1, 0)
    assert np.allclose(c0.viewproj, seq.keyframe(0, 0).viewproj, atol=1e-5)
    assert np.allclose(c4.viewproj, seq.keyframe(1, 0).viewproj, atol=1e-5)
    c2 = seq.client(0, 2)
    assert c2.alpha == 0.5 and c2.frames_per_anchor == 4
