// boost/optional.hpp stand-in: default/none construction, construction and
// assignment from a value, dereference and truth test.
#ifndef TT_SHIM_BOOST_OPTIONAL_HPP
#define TT_SHIM_BOOST_OPTIONAL_HPP
#include <stdexcept>
#include "none.hpp"
namespace boost {
template <typename T> class optional {
  public:
    optional() : set_(false), v_() {}
    optional(none_t) : set_(false), v_() {}
    optional(const T &v) : set_(true), v_(v) {}
    optional &operator=(const T &v) {
        set_ = true;
        v_ = v;
        return *this;
    }
    optional &operator=(none_t) {
        set_ = false;
        return *this;
    }
    const T &operator*() const {
        if (!set_)
            throw std::logic_error("dereferencing an empty boost::optional");
        return v_;
    }
    T &operator*() {
        if (!set_)
            throw std::logic_error("dereferencing an empty boost::optional");
        return v_;
    }
    explicit operator bool() const { return set_; }

  private:
    bool set_;
    T v_;
};
}
#endif
