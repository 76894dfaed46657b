// utils.h - the binary read helper cell/svodata.h uses.
#pragma once
#include <istream>

template <class T>
inline void read(std::istream& s, T& v) {
  s.read(reinterpret_cast<char*>(&v), sizeof(T));
}
