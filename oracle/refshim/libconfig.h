// Host stand-in for libconfig: reading "succeeds" with no settings, so the
// reference's readConfig keeps its defaults; the pin harness sets fields itself.
#pragma once
struct config_t { int dummy; };
struct config_setting_t { int dummy; };
enum { CONFIG_FALSE = 0, CONFIG_TRUE = 1 };
inline void config_init(config_t*) {}
inline void config_destroy(config_t*) {}
inline int config_read_file(config_t*, const char*) { return CONFIG_TRUE; }
inline const char* config_error_file(const config_t*) { return ""; }
inline int config_error_line(const config_t*) { return 0; }
inline const char* config_error_text(const config_t*) { return ""; }
inline config_setting_t* config_lookup(const config_t*, const char*) { return nullptr; }
inline config_setting_t* config_setting_lookup(config_setting_t*, const char*) { return nullptr; }
inline int config_setting_lookup_string(const config_setting_t*, const char*, const char**) { return CONFIG_FALSE; }
inline int config_setting_lookup_int(const config_setting_t*, const char*, int*) { return CONFIG_FALSE; }
inline int config_setting_lookup_float(const config_setting_t*, const char*, double*) { return CONFIG_FALSE; }
inline int config_setting_lookup_bool(const config_setting_t*, const char*, int*) { return CONFIG_FALSE; }
