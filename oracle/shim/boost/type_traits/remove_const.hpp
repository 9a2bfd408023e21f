// Compat shim (test infrastructure only): std:: type trait under the Boost name.
#ifndef ORACLE_SHIM_BOOST_TT_remove_const_HPP
#define ORACLE_SHIM_BOOST_TT_remove_const_HPP
#include <type_traits>
namespace boost { using std::remove_const; }
#endif
