// Compat shim (test infrastructure only): std:: type trait under the Boost name.
#ifndef ORACLE_SHIM_BOOST_TT_is_scalar_HPP
#define ORACLE_SHIM_BOOST_TT_is_scalar_HPP
#include <type_traits>
namespace boost { using std::is_scalar; }
#endif
