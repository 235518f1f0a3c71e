// gflags/gflags.h -- a small, header-only, gflags-compatible command-line
// flag parser for the Grus drop-in.
//
// The reference builds gflags from an empty git submodule (.gitmodules:1-3,
// CMakeLists.txt:13-16); it is not installed here, so this header supplies the
// part of its API the reference uses: DEFINE_/DECLARE_{string,bool,int32,
// int64,uint32,uint64,double} (include/app.cuh:11-31, samples/*/*.cu),
// gflags::ParseCommandLineFlags (include/app.cuh:37) and
// gflags::GetCommandLineFlagInfoOrDie(name).is_default (samples/bfs/bfs.cu:45).
// Accepted forms: --name=value, --name value, -name=value, --bool, --nobool.
// Like gflags, an unknown flag or a malformed value ends the program with a
// message (the command line is the user's interface, not the library's).
#ifndef GRUS_GFLAGS_SHIM_H
#define GRUS_GFLAGS_SHIM_H

#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace gflags {

struct CommandLineFlagInfo {
  std::string name;
  std::string type;
  std::string description;
  std::string current_value;
  std::string default_value;
  std::string filename;
  bool has_validator_fn = false;
  bool is_default = true;
  const void *flag_ptr = nullptr;
};

namespace shim {

enum class Kind { kBool, kInt32, kInt64, kUInt32, kUInt64, kDouble, kString };

struct Flag {
  Kind kind;
  void *ptr;
  std::string name, help, file, def;
  bool is_default = true;
};

inline std::map<std::string, Flag> &registry() {
  static std::map<std::string, Flag> r;
  return r;
}

inline const char *kind_name(Kind k) {
  switch (k) {
    case Kind::kBool: return "bool";
    case Kind::kInt32: return "int32";
    case Kind::kInt64: return "int64";
    case Kind::kUInt32: return "uint32";
    case Kind::kUInt64: return "uint64";
    case Kind::kDouble: return "double";
    default: return "string";
  }
}

inline std::string to_string(const Flag &f) {
  char buf[64];
  switch (f.kind) {
    case Kind::kBool: return *(bool *)f.ptr ? "true" : "false";
    case Kind::kInt32: std::snprintf(buf, sizeof buf, "%d", *(int32_t *)f.ptr); return buf;
    case Kind::kInt64: std::snprintf(buf, sizeof buf, "%lld", (long long)*(int64_t *)f.ptr); return buf;
    case Kind::kUInt32: std::snprintf(buf, sizeof buf, "%u", *(uint32_t *)f.ptr); return buf;
    case Kind::kUInt64: std::snprintf(buf, sizeof buf, "%llu", (unsigned long long)*(uint64_t *)f.ptr); return buf;
    case Kind::kDouble: std::snprintf(buf, sizeof buf, "%g", *(double *)f.ptr); return buf;
    default: return *(std::string *)f.ptr;
  }
}

// Parses `v` into the flag; false on a malformed value.
inline bool assign(Flag &f, const char *v) {
  char *end = nullptr;
  errno = 0;
  switch (f.kind) {
    case Kind::kBool: {
      const std::string s(v);
      if (s == "true" || s == "1" || s == "yes" || s == "t" || s == "y") *(bool *)f.ptr = true;
      else if (s == "false" || s == "0" || s == "no" || s == "f" || s == "n") *(bool *)f.ptr = false;
      else return false;
      return true;
    }
    case Kind::kInt32: { long long x = std::strtoll(v, &end, 0); if (*v == 0 || *end || x < INT32_MIN || x > INT32_MAX) return false; *(int32_t *)f.ptr = (int32_t)x; return true; }
    case Kind::kInt64: { long long x = std::strtoll(v, &end, 0); if (*v == 0 || *end) return false; *(int64_t *)f.ptr = x; return true; }
    case Kind::kUInt32: { unsigned long long x = std::strtoull(v, &end, 0); if (*v == 0 || *end || x > UINT32_MAX) return false; *(uint32_t *)f.ptr = (uint32_t)x; return true; }
    case Kind::kUInt64: { unsigned long long x = std::strtoull(v, &end, 0); if (*v == 0 || *end) return false; *(uint64_t *)f.ptr = x; return true; }
    case Kind::kDouble: { double x = std::strtod(v, &end); if (*v == 0 || *end) return false; *(double *)f.ptr = x; return true; }
    default: *(std::string *)f.ptr = v; return true;
  }
}

struct Registerer {
  Registerer(Kind k, void *ptr, const char *name, const char *help, const char *file) {
    Flag f{k, ptr, name, help ? help : "", file ? file : "", ""};
    f.def = to_string(f);
    registry()[name] = f;
  }
};

[[noreturn]] inline void die(const std::string &msg) {
  std::fprintf(stderr, "ERROR: %s\n", msg.c_str());
  std::exit(1);
}

}  // namespace shim

inline void SetUsageMessage(const std::string &) {}
inline void SetVersionString(const std::string &) {}
inline void ShutDownCommandLineFlags() {}

// Parses and (when remove_flags) removes the flags from argv, leaving the
// program name and positional arguments.  Returns the index of the first
// positional argument, as gflags does.
inline uint32_t ParseCommandLineFlags(int *argc, char ***argv, bool remove_flags) {
  auto &reg = shim::registry();
  std::vector<char *> keep;
  keep.push_back((*argv)[0]);
  bool only_positional = false;
  for (int i = 1; i < *argc; ++i) {
    char *arg = (*argv)[i];
    if (only_positional || arg[0] != '-' || arg[1] == 0) {
      keep.push_back(arg);
      continue;
    }
    if (std::strcmp(arg, "--") == 0) {
      only_positional = true;
      continue;
    }
    const char *body = arg + 1 + (arg[1] == '-');
    std::string name(body);
    const char *value = nullptr;
    const size_t eq = name.find('=');
    if (eq != std::string::npos) {
      value = body + eq + 1;
      name = name.substr(0, eq);
    }
    auto it = reg.find(name);
    bool negated = false;
    if (it == reg.end() && name.compare(0, 2, "no") == 0 && !value) {
      it = reg.find(name.substr(2));
      negated = it != reg.end() && it->second.kind == shim::Kind::kBool;
      if (!negated) it = reg.end();
    }
    if (it == reg.end()) shim::die("unknown command line flag '" + name + "'");
    shim::Flag &f = it->second;
    if (negated) {
      *(bool *)f.ptr = false;
    } else if (f.kind == shim::Kind::kBool && !value) {
      *(bool *)f.ptr = true;
    } else {
      if (!value) {
        if (i + 1 >= *argc) shim::die("flag '" + name + "' is missing its argument");
        value = (*argv)[++i];
      }
      if (!shim::assign(f, value)) shim::die("illegal value '" + std::string(value) + "' for flag '" + name + "'");
    }
    f.is_default = false;
  }
  if (remove_flags) {
    for (size_t k = 0; k < keep.size(); ++k) (*argv)[k] = keep[k];
    *argc = (int)keep.size();
    return 1;
  }
  return (uint32_t)*argc;
}

inline bool GetCommandLineFlagInfo(const char *name, CommandLineFlagInfo *out) {
  auto &reg = shim::registry();
  auto it = reg.find(name);
  if (it == reg.end()) return false;
  const shim::Flag &f = it->second;
  out->name = f.name;
  out->type = shim::kind_name(f.kind);
  out->description = f.help;
  out->current_value = shim::to_string(f);
  out->default_value = f.def;
  out->filename = f.file;
  out->is_default = f.is_default;
  out->flag_ptr = f.ptr;
  return true;
}

inline CommandLineFlagInfo GetCommandLineFlagInfoOrDie(const char *name) {
  CommandLineFlagInfo info;
  if (!GetCommandLineFlagInfo(name, &info)) shim::die(std::string("flag '") + name + "' does not exist");
  return info;
}

// Sets a flag by name as if from the command line; returns "" if unknown.
inline std::string SetCommandLineOption(const char *name, const char *value) {
  auto &reg = shim::registry();
  auto it = reg.find(name);
  if (it == reg.end() || !shim::assign(it->second, value)) return "";
  it->second.is_default = false;
  return std::string(name) + " set to " + value + "\n";
}

}  // namespace gflags

namespace google = gflags;

#define GRUS_GF_DEFINE(ns, type, kind, name, val, help)                          \
  namespace ns {                                                                 \
  type FLAGS_##name = val;                                                       \
  static ::gflags::shim::Registerer grus_gf_reg_##name(                          \
      ::gflags::shim::Kind::kind, &FLAGS_##name, #name, help, __FILE__);         \
  }                                                                              \
  using ns::FLAGS_##name

#define GRUS_GF_DECLARE(ns, type, name) \
  namespace ns {                        \
  extern type FLAGS_##name;             \
  }                                     \
  using ns::FLAGS_##name

#define DEFINE_bool(name, val, help) GRUS_GF_DEFINE(fLB, bool, kBool, name, val, help)
#define DEFINE_int32(name, val, help) GRUS_GF_DEFINE(fLI, int32_t, kInt32, name, val, help)
#define DEFINE_int64(name, val, help) GRUS_GF_DEFINE(fLI64, int64_t, kInt64, name, val, help)
#define DEFINE_uint32(name, val, help) GRUS_GF_DEFINE(fLU, uint32_t, kUInt32, name, val, help)
#define DEFINE_uint64(name, val, help) GRUS_GF_DEFINE(fLU64, uint64_t, kUInt64, name, val, help)
#define DEFINE_double(name, val, help) GRUS_GF_DEFINE(fLD, double, kDouble, name, val, help)
#define DEFINE_string(name, val, help) GRUS_GF_DEFINE(fLS, ::std::string, kString, name, val, help)

#define DECLARE_bool(name) GRUS_GF_DECLARE(fLB, bool, name)
#define DECLARE_int32(name) GRUS_GF_DECLARE(fLI, int32_t, name)
#define DECLARE_int64(name) GRUS_GF_DECLARE(fLI64, int64_t, name)
#define DECLARE_uint32(name) GRUS_GF_DECLARE(fLU, uint32_t, name)
#define DECLARE_uint64(name) GRUS_GF_DECLARE(fLU64, uint64_t, name)
#define DECLARE_double(name) GRUS_GF_DECLARE(fLD, double, name)
#define DECLARE_string(name) GRUS_GF_DECLARE(fLS, ::std::string, name)

#endif  // GRUS_GFLAGS_SHIM_H
