// Compat shim (test infrastructure only): BOOST_TYPEOF via decltype.  An alias
// template keeps the expansion valid inside dependent contexts without
// `typename`.
#ifndef ORACLE_SHIM_BOOST_TYPEOF_HPP
#define ORACLE_SHIM_BOOST_TYPEOF_HPP
#include <cstddef>
#include <type_traits>
template <typename T> using oracle_shim_decay_t = typename std::decay<T>::type;
#define BOOST_TYPEOF(e) oracle_shim_decay_t<decltype(e)>
#define BOOST_TYPEOF_TPL(e) oracle_shim_decay_t<decltype(e)>
#define BOOST_AUTO(v, e) auto v = e
#define BOOST_TYPEOF_REGISTER_TYPE(t)
#define BOOST_TYPEOF_REGISTER_TEMPLATE(t, n)
#define BOOST_TYPEOF_INCREMENT_REGISTRATION_GROUP() <cstddef>
#endif
