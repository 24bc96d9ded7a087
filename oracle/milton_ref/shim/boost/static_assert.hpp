/* Stand-in for Boost's static assertion when the reference's accel sources are compiled as a
 * test oracle (Boost is not installed): the C++11 keyword does the same check. */
#ifndef MILTON_REF_SHIM_STATIC_ASSERT_HPP_
#define MILTON_REF_SHIM_STATIC_ASSERT_HPP_
#define BOOST_STATIC_ASSERT(x) static_assert((x), #x)
#endif
