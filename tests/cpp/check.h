// Minimal check macros for the C++ API tests (the reference uses Boost.Test).
#pragma once
#include <cstdio>
#include <cstdlib>

static int g_failures = 0;
static int g_checks = 0;

#define CHECK_EQUAL(a, b)                                                              \
  do {                                                                                 \
    ++g_checks;                                                                        \
    if (!((a) == (b))) {                                                               \
      ++g_failures;                                                                    \
      std::printf("FAIL %s:%d: %s == %s\n", __FILE__, __LINE__, #a, #b);               \
    }                                                                                  \
  } while (0)

#define CHECK_THROW(expr, ex)                                                          \
  do {                                                                                 \
    ++g_checks;                                                                        \
    bool thrown_ = false;                                                              \
    try { expr; } catch (const ex&) { thrown_ = true; }                                \
    if (!thrown_) { ++g_failures; std::printf("FAIL %s:%d: %s did not throw\n", __FILE__, __LINE__, #expr); } \
  } while (0)

#define CHECK_NO_THROW(expr)                                                           \
  do {                                                                                 \
    ++g_checks;                                                                        \
    try { expr; } catch (...) { ++g_failures; std::printf("FAIL %s:%d: %s threw\n", __FILE__, __LINE__, #expr); } \
  } while (0)

#define TEST_MAIN_END()                                                                \
  std::printf("%d checks, %d failures\n", g_checks, g_failures);                      \
  return g_failures ? 1 : 0;
