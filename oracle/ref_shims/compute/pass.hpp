// Minimal restatement of wslam::compute::Pass (compute/include/compute/pass.hpp:19-27)
// so the reference matcher compiles without Dawn.  Test infrastructure.
#pragma once
#include <optional>
#include <string>
namespace wslam::compute {
class Pass {
   public:
    Pass() = default;
    virtual ~Pass() = default;
    [[nodiscard]] virtual std::string getId() const = 0;
    [[nodiscard]] virtual std::optional<std::string> initialize() = 0;
    [[nodiscard]] virtual std::optional<std::string> execute() = 0;
};
}  // namespace wslam::compute
