// Minimal stand-in for boost::lexical_cast used only to compile the reference
// headers in this container (parsing numbers out of Matrix-Market lines).
#pragma once
#include <sstream>
#include <string>
#include <stdexcept>
namespace boost {
template <typename Target, typename Source>
Target lexical_cast(const Source& s) {
    std::istringstream in(s);
    Target t{};
    in >> t;
    if (in.fail()) throw std::runtime_error("lexical_cast: bad input");
    return t;
}
}  // namespace boost
