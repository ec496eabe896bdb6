"""Error behaviour of the Python mirror of the reference classes (no GPU): the reference's own argument
checks, kept with their quirks, and the explicit refusals of modes the GPU engine does not implement."""
import numpy as np
import pytest

from pachydermacoustic_universal_gb300 import simulation as sim


def test_material_and_scattering_take_eight_bands():
    with pytest.raises(ValueError):
        sim.Basic_Material([0.1] * 7)
    with pytest.raises(ValueError):
        sim.Lambert_Scattering([0.2] * 9)
    assert sim.Basic_Material([0.1] * 8).Coefficient_A_Broad(3) == pytest.approx(0.1)


def _box_model():
    """One object: the six faces of a 2 x 2 x 2 m box as quads."""
    c = np.array([[x, y, z] for x in (0, 2) for y in (0, 2) for z in (0, 2)], dtype=np.float64)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    return [[c[list(f)] for f in faces]]


def test_construct_checks_codes_as_the_reference_does():
    """Polygon_Scene.Construct throws only when BOTH the material and the scattering lists miss the
    object count (Classes_Scenes.cs:449 joins the two tests with &&)."""
    model = _box_model()
    mat, scat = sim.Basic_Material([0.1] * 8), sim.Lambert_Scattering([0.2] * 8)
    s = sim.Polygon_Scene()
    with pytest.raises(ValueError):
        s.Construct(model, [], [])
    s.Construct(model, [mat], [scat, scat])  # one list right: accepted, as in the reference
    assert s.Valid and s.Count() == 6


def test_partition_needs_a_constructed_scene():
    with pytest.raises(RuntimeError):
        sim.Polygon_Scene().partition()


def test_modes_the_engine_does_not_implement_are_refused():
    with pytest.raises(NotImplementedError):
        sim.Source([120.0] * 8, (1.0, 1.0, 1.0), Third_Octave=True)
    with pytest.raises(NotImplementedError):
        sim.Direct_Sound(None, None, None, [0, 7], ScreenCalc=True)
    with pytest.raises(NotImplementedError):
        sim.IR_Construction.ETCurve(None, object(), None, 1000.0, 1000, 0, 0, False)
