// Test stand-in for wslam/include/wslam/common.hpp: the constants, keys and
// AnyBag members the adapter passes use (the real header needs Dawn).
#pragma once
#include <any>
#include <cstdint>
#include <optional>
#include <string>
#include <unordered_map>

class AnyBag {
   public:
    template <typename V>
    void set(const std::string& key, V&& value) {
        data_[key] = std::make_any<std::decay_t<V>>(std::forward<V>(value));
    }
    template <typename T>
    std::optional<T*> getPtr(const std::string& key) {
        auto it = data_.find(key);
        if (it == data_.end()) return std::nullopt;
        T* p = std::any_cast<T>(&it->second);
        if (!p) return std::nullopt;
        return p;
    }
    template <typename T>
    std::optional<T> take(const std::string& key) {
        auto it = data_.find(key);
        if (it == data_.end()) return std::nullopt;
        T* p = std::any_cast<T>(&it->second);
        if (!p) return std::nullopt;
        T v = std::move(*p);
        data_.erase(it);
        return v;
    }
    bool has(const std::string& key) const { return data_.count(key) != 0; }

   private:
    std::unordered_map<std::string, std::any> data_;
};

namespace wslam {
namespace GPUConst {
constexpr uint32_t levels_of_detail = 6;
}
namespace ResourceIdentifier {
inline std::string GetFrameName(uint32_t i) { return "res:frame:" + std::to_string(i) + ":lod:0"; }
inline std::string GetFeatureSetName(size_t k) { return "gen:feat:-" + std::to_string(k); }
inline const std::string MatchedFeaturesName = "gen:feat:match";
inline const std::string FeatureReferenceAdvanceName = "gen:feat:refadv";
}  // namespace ResourceIdentifier
}  // namespace wslam
