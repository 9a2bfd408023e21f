// Compat shim (test infrastructure only): declaration only; no tracker code
// path instantiates it.
#ifndef ORACLE_SHIM_BOOST_TT_FUNCTION_TRAITS_HPP
#define ORACLE_SHIM_BOOST_TT_FUNCTION_TRAITS_HPP
namespace boost { template <typename F> struct function_traits; }
#endif
