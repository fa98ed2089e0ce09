"""The section timer of the reference's Python surface (gstex_cuda/timer.py):
same methods and printed format; host wall-clock timing on CPU."""
import time

from gstex_cuda_gb300.timer import Timer


def test_timer_accumulates_and_dumps(capsys):
    t = Timer(cuda_support=False)
    for _ in range(2):
        t.start("render")
        time.sleep(0.01)
        t.stop()
        t.lap()
    t.start("dropped")  # started, never stopped: counts nothing
    t.start("project")
    t.stop()
    t.dump()
    out = capsys.readouterr().out.splitlines()
    assert [line.split("\t")[0] for line in out] == ["render", "dropped", "project", "TOTAL"]
    render = float(out[0].split("\t")[1])
    assert render >= 20.0 and float(out[1].split("\t")[1]) == 0.0
    assert abs(float(out[3].split("\t")[1]) - sum(float(line.split("\t")[1]) for line in out[:3])) < 1e-2
    assert t.laps == 2


def test_disabled_timer_does_nothing(capsys):
    t = Timer(disabled=True)
    t.start("a")
    t.stop()
    t.dump()
    assert capsys.readouterr().out == "" and t.times == {}
