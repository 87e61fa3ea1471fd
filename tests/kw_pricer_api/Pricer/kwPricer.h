// A minimal stand-in for the reference's pricer interface, written for the tests of
// this repository so that the kw::Pricer subclasses of the integration guide (the
// ones a maintainer of the reference would add) can be compiled and run where the
// reference's sources are absent.  It declares only what those subclasses use, with the signatures of
//   kw::Error                 src/Core/kwTypes.h:15     (std::string, empty = success)
//   kw::Option                src/Core/kwAsset.h:12-22  (56-byte record)
//   kw::Config::get / set     src/Core/kwConfig.h:21-73 (typed maps: real, integer, text)
//   kw::Pricer::init / price  src/Pricer/kwPricer.h:12-22
// TEST INFRASTRUCTURE ONLY.
#pragma once

#include <concepts>
#include <cstdint>
#include <map>
#include <string>
#include <string_view>
#include <type_traits>
#include <vector>

namespace kw {

using Error = std::string;
using f64 = double;
using i64 = std::int64_t;
using u8 = std::uint8_t;
using i8 = std::int8_t;

struct Option {
    f64 t;  // maturity, years
    f64 k;  // strike
    f64 z;  // volatility
    f64 r;  // rate
    f64 q;  // dividend yield
    f64 s;  // spot
    u8 e;   // 1 American, 0 European
    i8 w;   // +1 call, -1 put
};

// Keys live in one of three typed tables; a lookup uses the table of the default
// value's type and returns the default for a key the table lacks.
class Config {
    std::map<std::string, f64> real_;
    std::map<std::string, i64> integer_;
    std::map<std::string, std::string> text_;

public:
    template <std::floating_point T>
    f64 get(const std::string& key, T fallback) const
    {
        auto it = real_.find(key);
        return it == real_.end() ? fallback : it->second;
    }
    template <std::integral T>
    i64 get(const std::string& key, T fallback) const
    {
        auto it = integer_.find(key);
        return it == integer_.end() ? fallback : it->second;
    }
    template <class T>
        requires std::is_convertible_v<T, std::string_view>
    std::string get(const std::string& key, const T& fallback) const
    {
        auto it = text_.find(key);
        return it == text_.end() ? std::string(fallback) : it->second;
    }

    template <std::floating_point T>
    void set(const std::string& key, T v)
    {
        real_[key] = v;
    }
    template <std::integral T>
    void set(const std::string& key, T v)
    {
        integer_[key] = v;
    }
    template <class T>
        requires std::is_convertible_v<T, std::string_view>
    void set(const std::string& key, const T& v)
    {
        text_[key] = std::string(v);
    }
};

class Pricer {
public:
    virtual ~Pricer() = default;
    virtual Error init(const Config& config) = 0;
    virtual Error price(const std::vector<Option>& assets, std::vector<double>& prices) = 0;
};

}  // namespace kw
