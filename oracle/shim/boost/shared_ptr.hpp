// Compat shim (test infrastructure only): maps the one Boost smart pointer the
// reference uses onto std::shared_ptr so the reference CPU tracker compiles
// without Boost.
#ifndef ORACLE_SHIM_BOOST_SHARED_PTR_HPP
#define ORACLE_SHIM_BOOST_SHARED_PTR_HPP
#include <memory>
namespace boost { using std::shared_ptr; }
#endif
