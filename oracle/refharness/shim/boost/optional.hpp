// boost::optional stand-in for compiling the reference's renderer_bdpt.cpp
// without boost: the subset it uses (construction from a value or
// boost::none, get(), operator bool, *, ->) on top of std::experimental.
#pragma once
#include <experimental/optional>

namespace boost {

template <class T>
class optional : public std::experimental::optional<T>
{
    using base = std::experimental::optional<T>;

public:
    using base::base;
    optional() = default;
    optional(const base& b) : base(b) {}
    T& get() { return **this; }
    const T& get() const { return **this; }
};

constexpr std::experimental::nullopt_t none = std::experimental::nullopt;

}  // namespace boost
