// boost/lexical_cast.hpp stand-in: whole-string numeric conversion that
// throws bad_lexical_cast on any leftover or missing characters.
#ifndef TT_SHIM_BOOST_LEXICAL_CAST_HPP
#define TT_SHIM_BOOST_LEXICAL_CAST_HPP
#include <sstream>
#include <typeinfo>
#include <stdexcept>
#include <string>
namespace boost {
class bad_lexical_cast : public std::bad_cast {
  public:
    const char *what() const noexcept override {
        return "bad lexical cast: source type value could not be interpreted "
               "as target";
    }
};
template <typename T> T lexical_cast(const std::string &s) {
    if (s.empty() || s[0] == '-' || s[0] == '+' || s[0] == ' ')
        throw bad_lexical_cast();
    std::istringstream in(s);
    T v;
    in >> v;
    if (in.fail() || !in.eof())
        throw bad_lexical_cast();
    return v;
}
}
#endif
