// Minimal stand-in for <gtest/gtest.h> so that pwm's test/util/util.hpp (which
// only needs the assertion macros) compiles into the reference driver.  The
// googletest submodule of the reference is empty in this environment.
#pragma once
#include <sstream>
#include <string>
namespace pwmref_stub { struct sink { template <class T> sink& operator<<(const T&) { return *this; } }; }
#define ASSERT_EQ(a, b) if (!((a) == (b))) pwmref_stub::sink()
#define EXPECT_EQ(a, b) if (!((a) == (b))) pwmref_stub::sink()
