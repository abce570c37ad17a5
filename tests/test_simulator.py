"""CPU checks of the frame driver (swc.Simulator, the reference's Simulator) with a
scripted simulation: the substep rule of Simulator::advanceTimeBySteps
(Cores/Physics/Simulator.cpp:103-128), the frame files of Simulate
(Simulator.cpp:14-71, 79-91) and the resume path."""
import math
import os

import pytest

from swc.simulator import Simulator, substep_schedule


class Scripted:
    """Simulation stand-in: getTimeStep returns the scripted values in turn."""

    def __init__(self, steps):
        self.steps = list(steps)
        self.calls = []

    def initialize(self):
        self.calls.append("initialize")

    def getTimeStep(self, frameRate, stepRate):
        return self.steps.pop(0) if len(self.steps) > 1 else self.steps[0]

    def advance(self, dt):
        self.calls.append(("advance", dt))

    def writeFrame(self, d, staticDraw=False):
        open(os.path.join(d, "particles.mesh"), "wb").close()

    def saveFrame(self, d):
        open(os.path.join(d, "particles.sav"), "wb").close()

    def loadFrame(self, d):
        self.calls.append(("loadFrame", os.path.basename(d)))

    def writeDescription(self, path):
        with open(path, "w") as f:
            f.write("dimension: 2\n")


def restated(target, steps):
    """The reference's loop, restated: the substeps of one frame."""
    t, out, i = 0.0, [], 0
    while True:
        dt = steps[min(i, len(steps) - 1)]
        i += 1
        if t + dt >= target:
            out.append(target - t)
            return out
        if t + 2 * dt >= target:
            dt = (target - t) / 2
        out.append(dt)
        t += dt


@pytest.mark.parametrize("steps", [[0.3], [0.4], [0.6], [1.5], [0.26, 0.3, 0.5], [0.1] * 20, [math.inf]])
def test_substep_rule(steps):
    sim = Simulator("unused", 1, 1, 1, 0.5, Scripted(steps))
    taken = sim.advanceTimeBySteps(1.0)
    assert taken == restated(1.0, steps)
    assert sum(taken) == pytest.approx(1.0, abs=1e-15)


def test_last_two_substeps_share_the_rest():
    # 0.45: after one step two more would overshoot, so the remaining 0.55 is split
    assert Simulator("unused", 1, 1, 1, 0.5, Scripted([0.45])).advanceTimeBySteps(1.0) == \
        pytest.approx([0.45, 0.275, 0.275], rel=1e-15)
    assert substep_schedule(0.0, 1.0, 2.0) == (1.0, True)
    assert substep_schedule(0.0, 1.0, 0.5) == (0.5, False)  # time + 2 dt reaches the target: half of the rest
    assert substep_schedule(0.0, 1.0, 0.4) == (0.4, False)


@pytest.mark.parametrize("bad", [0.0, -1e-3, math.nan])
def test_step_that_cannot_advance_raises(bad):
    with pytest.raises(ValueError):
        Simulator("unused", 1, 1, 1, 0.5, Scripted([bad])).advanceTimeBySteps(1.0)


def test_simulate_writes_frames_and_resumes(tmp_path):
    out = tmp_path / "run"
    sim = Scripted([0.004])
    Simulator(str(out), 0, 3, 100, 0.5, sim).Simulate()
    assert sim.calls[0] == "initialize"
    for f in range(3):
        assert (out / str(f) / "particles.sav").exists() and (out / str(f) / "particles.mesh").exists()
    assert (out / "end_frame.txt").read_text().strip() == "3"
    assert (out / "description.yaml").read_text().startswith("dimension: 2")
    # 1/100 per frame in steps of 0.004: 0.004, then the rest 0.006 split evenly
    adv = [c[1] for c in sim.calls if c[0] == "advance"]
    assert adv == pytest.approx([0.004, 0.003, 0.003] * 2, rel=1e-12)
    # resume: load frame 2, run frame 3
    sim2 = Scripted([0.02])
    Simulator(str(out), 3, 4, 100, 0.5, sim2).Simulate()
    assert sim2.calls[0] == ("loadFrame", "2") and "initialize" not in sim2.calls
    assert (out / "end_frame.txt").read_text().strip() == "4"
    with pytest.raises(FileNotFoundError):
        Simulator(str(out), 9, 10, 100, 0.5, Scripted([0.02])).Simulate()
