// Minimal stand-in for the better-enums BETTER_ENUM macro: an enum wrapper
// with unary + on enumerators, _to_integral, _to_string and
// _from_string_nothrow (the subset the reference's model headers use).
#pragma once
#include <cstring>
#include <string>
namespace be_shim
{
inline std::string
nth_name(const char * names, int n)
{
  std::string s(names), tok;
  int         k = 0;
  size_t      i = 0;
  while (i <= s.size())
  {
    size_t j = s.find(',', i);
    if (j == std::string::npos)
      j = s.size();
    tok = s.substr(i, j - i);
    size_t a = tok.find_first_not_of(" \t\n"), b = tok.find_last_not_of(" \t\n");
    tok = a == std::string::npos ? "" : tok.substr(a, b - a + 1);
    if (k == n)
      return tok;
    ++k;
    i = j + 1;
  }
  return "";
}
} // namespace be_shim
#define BETTER_ENUM(Name, Type, ...)                                                             \
  struct Name                                                                                    \
  {                                                                                              \
    enum _enumerated : Type                                                                      \
    {                                                                                            \
      __VA_ARGS__                                                                                \
    };                                                                                           \
    _enumerated _value;                                                                          \
    constexpr Name(_enumerated v)                                                                \
      : _value(v)                                                                                \
    {}                                                                                           \
    constexpr operator _enumerated() const { return _value; }                                    \
    constexpr Type _to_integral() const { return static_cast<Type>(_value); }                    \
    std::string _to_string() const { return be_shim::nth_name(#__VA_ARGS__, (int)_value); }     \
    struct _opt                                                                                  \
    {                                                                                            \
      bool        ok;                                                                            \
      _enumerated v;                                                                             \
      explicit operator bool() const { return ok; }                                              \
      Name operator*() const { return Name(v); }                                                 \
    };                                                                                           \
    static _opt _from_string_nothrow(const char * s)                                             \
    {                                                                                            \
      for (int i = 0; i < 64; ++i)                                                               \
      {                                                                                          \
        std::string n = be_shim::nth_name(#__VA_ARGS__, i);                                      \
        if (n.empty())                                                                           \
          break;                                                                                 \
        if (n == s)                                                                              \
          return { true, static_cast<_enumerated>(i) };                                          \
      }                                                                                          \
      return { false, static_cast<_enumerated>(0) };                                             \
    }                                                                                            \
  };                                                                                             \
  inline constexpr Name operator+(Name::_enumerated e) { return Name(e); }
