// Compat shim (test infrastructure only): array-owning shared pointer.
#ifndef ORACLE_SHIM_BOOST_SHARED_ARRAY_HPP
#define ORACLE_SHIM_BOOST_SHARED_ARRAY_HPP
#include <memory>
#include <cstddef>
namespace boost {
template <typename T>
class shared_array {
 public:
  shared_array() {}
  explicit shared_array(T* p) : p_(p, std::default_delete<T[]>()) {}
  template <typename D> shared_array(T* p, D d) : p_(p, d) {}
  T* get() const { return p_.get(); }
  T& operator[](std::ptrdiff_t i) const { return p_.get()[i]; }
  void reset() { p_.reset(); }
  void reset(T* p) { p_.reset(p, std::default_delete<T[]>()); }
  void swap(shared_array& o) { p_.swap(o.p_); }
  explicit operator bool() const { return bool(p_); }
 private:
  std::shared_ptr<T> p_;
};
}
#endif
