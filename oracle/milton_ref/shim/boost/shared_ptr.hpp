/* Stand-in for boost::shared_ptr on top of std::shared_ptr. */
#ifndef MILTON_REF_SHIM_SHARED_PTR_HPP_
#define MILTON_REF_SHIM_SHARED_PTR_HPP_
#include <memory>
namespace boost {
using std::shared_ptr;
using std::dynamic_pointer_cast;
using std::static_pointer_cast;
}  // namespace boost
#endif
