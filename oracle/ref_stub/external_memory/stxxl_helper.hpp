// Minimal stand-in for pwm's external_memory/stxxl_helper.hpp so that
// include/util/alphabet_util.hpp compiles into the reference driver without
// STXXL (its submodule is empty in this environment).  Only the names of the
// STXXL-backed types are declared: the driver instantiates the in-memory
// reduce_alphabet(std::vector&) only, never the overload that streams
// through these types.
#pragma once
template <typename T> class stxxlvector;
template <typename T> class stxxlreader;
template <typename T> class stxxlwriter;
