// Minimal restatement of the stage sentinel (compute/include/compute/stage.hpp:15).
// Test infrastructure.
#pragma once
#include <string>
#include "compute/pass.hpp"
namespace wslam::compute {
inline const std::string kStageStopExecution = "STAGE_STOP";
}
