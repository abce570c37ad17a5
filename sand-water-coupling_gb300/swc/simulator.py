"""Frame driver of the reference's Simulator (Cores/Physics/Simulator.{h,cpp}) for the
GPU simulations of this package (DualParticleSphLiquid, DEMParticleSand).

    Simulator(outputDir, beginFrame, endFrame, frameRate, stepRate, simulation).Simulate()

runs frames [beginFrame, endFrame) of 1 / frameRate seconds each, every frame
substepped as Simulator::advanceTimeBySteps does (Simulator.cpp:103-128): the
step is the simulation's getTimeStep(frameRate, stepRate) (for the liquid
stepRate * 2 r / max |v|, a CFL number), cut to land on the frame time, and the
last two substeps of a frame share the remaining time evenly.  Frames are
written and saved into outputDir/<frame>/ with end_frame.txt after each
(Simulator.cpp:79-91); frame 0 is written after initialize together with
description.yaml (Simulator.cpp:19-42); a run with beginFrame > 0 resumes from the
saved frame beginFrame - 1 (Simulator.cpp:43-45; the simulations here restore
their full state on loadFrame, which the reference's resume skips).

One deliberate difference: a time step that is not positive (NaN, zero or
negative) raises ValueError, where the reference would loop without end.
"""
from __future__ import annotations

import os


def substep_schedule(time: float, target: float, dt: float):
    """One decision of Simulator::advanceTimeBySteps (Simulator.cpp:111-118): the step
    to take from `time` towards `target` given the simulation's step `dt`, and
    whether it ends the frame."""
    if time + dt >= target:
        return target - time, True
    if time + 2 * dt >= target:
        return (target - time) / 2, False
    return dt, False


class Simulator:
    def __init__(self, outputDir, beginFrame, endFrame, frameRate, stepRate, simulation, verbose=False):
        self.outputDir = str(outputDir)
        self.beginFrame = int(beginFrame)
        self.endFrame = int(endFrame)
        self.frameRate = int(frameRate)
        self.stepRate = float(stepRate)
        self.simulation = simulation
        self.verbose = verbose
        self.substeps = []  # (frame, dt) of every advance made by Simulate / advanceTimeBySteps

    def _log(self, msg):
        if self.verbose:
            print(msg, flush=True)

    def Simulate(self):
        """Simulator::Simulate (Simulator.cpp:14-71)."""
        sim = self.simulation
        if self.beginFrame == 0:
            self._log("[Initialize]")
            sim.initialize()
            os.makedirs(self.outputDir, exist_ok=True)
            self.writeAndSaveToFrameDirectory(0, staticDraw=True)
            sim.writeDescription(os.path.join(self.outputDir, "description.yaml"))
            self.beginFrame = 1
        else:
            self.loadFromFrameDirectory(self.beginFrame - 1)
        for frame in range(self.beginFrame, self.endFrame):
            self._log(f"** Simulate Frame {frame}...")
            self.advanceTimeBySteps(1.0 / self.frameRate, frame=frame)
            self.writeAndSaveToFrameDirectory(frame)

    def advanceTimeBySteps(self, targetTime, frame=None):
        """Simulator::advanceTimeBySteps (Simulator.cpp:103-128); returns the steps taken."""
        sim = self.simulation
        time = 0.0
        done = time >= targetTime
        taken = []
        while not done:
            dt = sim.getTimeStep(self.frameRate, self.stepRate)
            if not (dt > 0):
                raise ValueError(f"time step {dt!r} from getTimeStep: the frame cannot advance")
            dt, done = substep_schedule(time, targetTime, dt)
            sim.advance(dt)
            time += dt
            taken.append(dt)
            self.substeps.append((frame, dt))
        return taken

    def writeAndSaveToFrameDirectory(self, frame, staticDraw=False):
        """Simulator::writeAndSaveToFrameDirectory (Simulator.cpp:79-91)."""
        frame_dir = os.path.join(self.outputDir, str(frame))
        os.makedirs(frame_dir, exist_ok=True)
        self.simulation.writeFrame(frame_dir, staticDraw)
        self.simulation.saveFrame(frame_dir)
        with open(os.path.join(self.outputDir, "end_frame.txt"), "w") as f:
            f.write(f"{frame + 1}\n")

    def loadFromFrameDirectory(self, frame):
        """Simulator::loadFromFrameDirectory (Simulator.cpp:93-101)."""
        frame_dir = os.path.join(self.outputDir, str(frame))
        if not os.path.isdir(frame_dir):
            raise FileNotFoundError(f"Simulator: no output directory for frame {frame}")
        self.simulation.loadFrame(frame_dir)

