// The library's C entry points end in WAP_CATCH (a function-try-block
// handler): an exception from the host-side C++ behind them (an allocation of
// the job lists, tables and strings the library builds, a worker thread that
// cannot be started) becomes a status code instead of unwinding into a C or
// ctypes caller, which would terminate the process.
#pragma once
#include <new>

#include "wap/wap.h"

#define WAP_CATCH                      \
  catch (const std::bad_alloc &) {     \
    return WAP_ENOMEM;                 \
  }                                    \
  catch (...) {                        \
    return WAP_EHOST;                  \
  }
