// Compatibility shim (test infrastructure): logging macros.
#pragma once
#include <cstdio>

#define log_error(...) do { std::fprintf(stderr, "[error] " __VA_ARGS__); std::fputc('\n', stderr); } while (0)
#define log_warn(...)  do { std::fprintf(stderr, "[warn] " __VA_ARGS__); std::fputc('\n', stderr); } while (0)
#define log_info(...)  do { std::fprintf(stderr, "[info] " __VA_ARGS__); std::fputc('\n', stderr); } while (0)
#define log_debug(...) do { } while (0)
