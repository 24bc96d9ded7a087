/* Stand-in for the Boost.Random names the reference's Random.h declares, on top of <random>.
 * Used only to compile the reference's intersection sources as a CPU test oracle: the
 * ray queries it answers draw no random numbers. */
#ifndef MILTON_REF_SHIM_RANDOM_HPP_
#define MILTON_REF_SHIM_RANDOM_HPP_
#include <cmath>
#include <random>
#include <vector>
namespace boost {
using mt19937 = std::mt19937;
template <typename T = double> using uniform_real = std::uniform_real_distribution<T>;
template <typename T = int> using uniform_int = std::uniform_int_distribution<T>;
template <typename T = double> using normal_distribution = std::normal_distribution<T>;
template <typename T = double> using exponential_distribution = std::exponential_distribution<T>;
template <typename T = double> class uniform_on_sphere {
 public:
  typedef std::vector<T> result_type;
  explicit uniform_on_sphere(int dim = 2) : dim_(dim) {}
  template <typename E> std::vector<T> operator()(E &e) {
    std::vector<T> v(dim_);
    T n = 0;
    do {
      n = 0;
      for (auto &x : v) { x = nd_(e); n += x * x; }
    } while (n == 0);
    n = std::sqrt(n);
    for (auto &x : v) x /= n;
    return v;
  }
 private:
  int dim_;
  std::normal_distribution<T> nd_;
};
template <typename Engine, typename Dist> class variate_generator {
 public:
  variate_generator(Engine e, Dist d) : e_(e), d_(d) {}
  auto operator()() const { return d_(e_); }
  Dist &distribution() { return d_; }
 private:
  Engine e_;
  mutable Dist d_;
};
}  // namespace boost
#endif
