"""The usage tour (every kernel family once at moderate sizes) runs and its
results are finite."""
import pytest

pytestmark = pytest.mark.gpu


def test_tour_runs(capsys):
    from spsslangevinintegration_gb300 import tour

    tour.main()
    out = capsys.readouterr().out
    assert "tour done" in out
    assert "nan" not in out.lower()
    assert "finite True" in out
