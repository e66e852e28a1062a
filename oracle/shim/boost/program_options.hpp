// boost/program_options.hpp stand-in: only validation_error, which the
// functional parsers throw (c++/src/sinogram.cpp:61-63, circus.cpp:44-65).
#ifndef TT_SHIM_BOOST_PROGRAM_OPTIONS_HPP
#define TT_SHIM_BOOST_PROGRAM_OPTIONS_HPP
// (the real header pulls in <map>, <vector> and <string> for variables_map)
#include <map>
#include <stdexcept>
#include <string>
#include <vector>
namespace boost {
namespace program_options {
class validation_error : public std::logic_error {
  public:
    enum kind_t {
        multiple_values_not_allowed = 30,
        at_least_one_value_required,
        invalid_bool_value,
        invalid_option_value,
        invalid_option
    };
    validation_error(kind_t kind, const std::string &option_name = "",
                     const std::string &original_token = "")
        : std::logic_error("the argument ('" + original_token +
                           "') for option '" + option_name + "' is invalid"),
          kind_(kind) {}
    kind_t kind() const { return kind_; }

  private:
    kind_t kind_;
};
}
}
#endif
