// Autotuned choices (kernel variants, solve methods, panel widths), keyed by the device and the problem's size. They
// live for the process and, when a tuning file is set (pcbqs_gb300_tune_file, or the PCBQS_GB300_TUNE_FILE
// environment variable at the first lookup), are read from it once and written back after every new choice, so a
// later process on the same kind of device takes them without timing anything.
#pragma once
#include <string>

namespace pq {

// The remembered choice for `key` on the current device, or -1.
int tune_get(const std::string &key);
// Remembers `value` for `key` on the current device and rewrites the tuning file, if one is set.
void tune_put(const std::string &key, int value);

}  // namespace pq
