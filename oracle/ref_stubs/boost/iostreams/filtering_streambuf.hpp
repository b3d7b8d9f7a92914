/* Test infrastructure (oracle build only). Minimal stand-in for Boost
 * iostreams: the reference's gzip three-body readers
 * (src/ThreeBodyStorage_no2b.cc:569, src/ThreeBodyStorage_mono.cc:744) need
 * these names to compile; they are never called on the IMSRG(2) path. */
#pragma once
#include <istream>
namespace boost { namespace iostreams {
struct gzip_decompressor {};
struct filtering_istream : public std::istream {
  filtering_istream() : std::istream(nullptr) {}
  template <class T> void push(T&) {}
  template <class T> void push(const T&) {}
};
}}
