/* Forced-include shim for building the unmodified reference sources with a
 * current g++/glibc: glibc >= 2.34 makes SIGSTKSZ a runtime value, which the
 * vendored Catch header uses as an array bound, and json.hpp relies on
 * <cstdint> arriving transitively. Test infrastructure only. */
#pragma once
#include <signal.h>
#undef SIGSTKSZ
#define SIGSTKSZ 32768
#include <cstdint>
