// Test stand-in for the stage sentinel (compute/include/compute/stage.hpp:15).
#pragma once
#include <string>
#include "compute/pass.hpp"
namespace wslam::compute {
inline const std::string kStageStopExecution = "STAGE_STOP";
}
