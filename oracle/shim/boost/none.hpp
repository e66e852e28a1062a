// boost/none.hpp stand-in (the subset maleadt/tracetransform uses).
#ifndef TT_SHIM_BOOST_NONE_HPP
#define TT_SHIM_BOOST_NONE_HPP
namespace boost {
struct none_t {};
const none_t none = none_t();
}
#endif
