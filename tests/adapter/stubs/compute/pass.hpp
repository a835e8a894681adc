// Test stand-in for compute/include/compute/pass.hpp:19-27.
#pragma once
#include <optional>
#include <string>
namespace wslam::compute {
class Pass {
   public:
    virtual ~Pass() = default;
    [[nodiscard]] virtual std::string getId() const = 0;
    [[nodiscard]] virtual std::optional<std::string> initialize() = 0;
    [[nodiscard]] virtual std::optional<std::string> execute() = 0;
};
}  // namespace wslam::compute
