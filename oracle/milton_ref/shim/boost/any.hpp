/* Stand-in for boost::any on top of std::any (same value semantics; empty() added). */
#ifndef MILTON_REF_SHIM_ANY_HPP_
#define MILTON_REF_SHIM_ANY_HPP_
#include <any>
#include <typeinfo>
#include <utility>
namespace boost {
class any : public std::any {
 public:
  any() = default;
  any(const any &) = default;
  any(any &&) = default;
  template <typename T, typename = std::enable_if_t<!std::is_same_v<std::decay_t<T>, any>>>
  any(T &&v) : std::any(std::forward<T>(v)) {}
  any &operator=(const any &) = default;
  any &operator=(any &&) = default;
  template <typename T, typename = std::enable_if_t<!std::is_same_v<std::decay_t<T>, any>>>
  any &operator=(T &&v) {
    std::any::operator=(std::forward<T>(v));
    return *this;
  }
  bool empty() const { return !has_value(); }
};
using bad_any_cast = std::bad_any_cast;
template <typename T> T any_cast(any &a) { return std::any_cast<T>(static_cast<std::any &>(a)); }
template <typename T> T any_cast(const any &a) { return std::any_cast<T>(static_cast<const std::any &>(a)); }
template <typename T> T *any_cast(any *a) { return std::any_cast<T>(static_cast<std::any *>(a)); }
template <typename T> const T *any_cast(const any *a) { return std::any_cast<T>(static_cast<const std::any *>(a)); }
}  // namespace boost
#endif
