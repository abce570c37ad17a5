// Simulator.hpp -- C++20 frame driver with the behaviour of PhysX::Simulator
// (Cores/Physics/Simulator.{h,cpp} of skytang0205/sand-water-coupling) for the GB300
// simulations of this library (swc::DualParticleSphLiquid<Dim>, swc::DEMParticleSand<Dim>)
// or any class with the same Simulation methods.
//
//   Simulate()                    Simulator.cpp:14-71: initialize + frame 0 + description.yaml
//                                 when beginFrame == 0, else resume from the saved frame
//                                 beginFrame - 1; then one frame of 1 / frameRate per loop.
//   advanceTimeBySteps(target)    Simulator.cpp:103-128: dt = getTimeStep(frameRate, stepRate)
//                                 cut to land on the target; the last two substeps share the
//                                 remaining time evenly.
//   writeAndSaveToFrameDirectory  Simulator.cpp:79-91 (frame files and end_frame.txt).
//
// A time step that is not positive (NaN, zero or negative) throws std::runtime_error
// where the reference would loop without end.
#pragma once

#include <filesystem>
#include <fstream>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace swc {

template<class Sim> class Simulator {
public:
    Simulator(std::string outputDir, unsigned beginFrame, unsigned endFrame, unsigned frameRate, double stepRate,
              Sim * simulation)
        : outputDir_(std::move(outputDir)), beginFrame_(beginFrame), endFrame_(endFrame), frameRate_(frameRate),
          stepRate_(stepRate), sim_(simulation) {}

    void Simulate() {
        if (beginFrame_ == 0) {
            sim_->initialize();
            std::filesystem::create_directories(outputDir_);
            writeAndSaveToFrameDirectory(0, true);
            if constexpr (requires(Sim & s, const std::string & p) { s.writeDescription(p); })
                sim_->writeDescription(outputDir_ + "/description.yaml");
            beginFrame_ = 1;
        } else {
            loadFromFrameDirectory(beginFrame_ - 1);
        }
        for (unsigned frame = beginFrame_; frame < endFrame_; frame++) {
            advanceTimeBySteps(1.0 / frameRate_);
            writeAndSaveToFrameDirectory(frame);
            if (onFrame) onFrame(frame);
        }
    }

    // Returns the substeps taken.
    std::vector<double> advanceTimeBySteps(double targetTime) {
        std::vector<double> taken;
        double time = 0;
        bool   done = time >= targetTime;
        while (!done) {
            double dt = sim_->getTimeStep(frameRate_, stepRate_);
            if (!(dt > 0)) throw std::runtime_error("Simulator: getTimeStep returned a step that is not positive");
            if (time + dt >= targetTime) {
                dt   = targetTime - time;
                done = true;
            } else if (time + 2 * dt >= targetTime) {
                dt = (targetTime - time) / 2;
            }
            sim_->advance(dt);
            time += dt;
            taken.push_back(dt);
            if (onSubstep) onSubstep(dt);
        }
        return taken;
    }

    void writeAndSaveToFrameDirectory(unsigned frame, bool staticDraw = false) {
        const std::string frameDir = outputDir_ + "/" + std::to_string(frame);
        std::filesystem::create_directories(frameDir);
        sim_->writeFrame(frameDir, staticDraw);
        sim_->saveFrame(frameDir);
        std::ofstream(outputDir_ + "/end_frame.txt") << frame + 1 << "\n";
    }

    void loadFromFrameDirectory(unsigned frame) {
        const std::string frameDir = outputDir_ + "/" + std::to_string(frame);
        if (!std::filesystem::exists(frameDir))
            throw std::runtime_error("Simulator: no output directory for frame " + std::to_string(frame));
        sim_->loadFrame(frameDir);
    }

    // Optional observers (progress output, tests).
    std::function<void(double)>   onSubstep;
    std::function<void(unsigned)> onFrame;

private:
    std::string outputDir_;
    unsigned    beginFrame_, endFrame_, frameRate_;
    double      stepRate_;
    Sim *       sim_;
};

}  // namespace swc
