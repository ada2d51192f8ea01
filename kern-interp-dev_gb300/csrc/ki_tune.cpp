// The autotuner's table (see ki_tune.h): one atomic choice per (knob,
// bucket), read by every launch site, replaced whole by tune_from_json.
#include "ki_tune.h"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace ki {

namespace {

std::atomic<int> g_table[kTuneKnobs][kTuneBuckets];
std::atomic<int> g_force[kTuneKnobs];
std::atomic<bool> g_recording{false};

struct Init {
  Init() {
    for (auto& row : g_table)
      for (auto& c : row) c.store(-1);
    for (auto& f : g_force) f.store(-1);
  }
} g_init;

const char* const kKnobNames[kTuneKnobs] = {"id", "schur", "sweep"};

int clampi(int v, int lo, int hi) { return std::max(lo, std::min(hi, v)); }

}  // namespace

int id_bucket(bool fp64, int group, int n_max) {
  return (fp64 ? 256 : 0) + clampi(group, 0, 3) * 64 + clampi((n_max + 31) / 32, 0, 63);
}

int schur_bucket(bool fp64, int r_max, int per_sm) {
  return (fp64 ? 256 : 0) + clampi((r_max + 31) / 32, 0, 31) * 8 + clampi(per_sm, 0, 7);
}

int sweep_bucket(bool fp64, int n_max) { return (fp64 ? 256 : 0) + clampi((n_max + 31) / 32, 0, 255); }

int tune_choice(int knob, int bucket) {
  if (knob < 0 || knob >= kTuneKnobs || bucket < 0 || bucket >= kTuneBuckets) return -1;
  const int f = g_force[knob].load(std::memory_order_relaxed);
  if (f >= 0) return f;
  return g_table[knob][bucket].load(std::memory_order_relaxed);
}

void tune_set(int knob, int bucket, int choice) {
  if (knob < 0 || knob >= kTuneKnobs || bucket < 0 || bucket >= kTuneBuckets)
    throw std::invalid_argument("tune: knob or bucket out of range");
  if (choice < -1 || choice >= kTuneCandidates[knob])
    throw std::invalid_argument("tune: candidate out of range");
  g_table[knob][bucket].store(choice);
}

void tune_clear() {
  for (auto& row : g_table)
    for (auto& c : row) c.store(-1);
}

void tune_force(int knob, int choice) {
  if (knob < 0 || knob >= kTuneKnobs) throw std::invalid_argument("tune: knob out of range");
  g_force[knob].store(choice);
}

bool tune_recording() { return g_recording.load(std::memory_order_relaxed); }
void tune_set_recording(bool on) { g_recording.store(on); }

std::string tune_stage(int knob, int bucket) {
  return std::string("tune:") + kKnobNames[knob] + ":" + std::to_string(bucket);
}

bool tune_parse_stage(const std::string& s, int* knob, int* bucket) {
  if (s.compare(0, 5, "tune:") != 0) return false;
  const size_t c = s.find(':', 5);
  if (c == std::string::npos) return false;
  const std::string name = s.substr(5, c - 5);
  for (int k = 0; k < kTuneKnobs; k++)
    if (name == kKnobNames[k]) {
      *knob = k;
      *bucket = std::atoi(s.c_str() + c + 1);
      return true;
    }
  return false;
}

std::string tune_to_json() {
  std::string out = "{";
  bool first = true;
  for (int k = 0; k < kTuneKnobs; k++)
    for (int b = 0; b < kTuneBuckets; b++) {
      const int c = g_table[k][b].load();
      if (c < 0) continue;
      out += first ? "" : ", ";
      first = false;
      out += "\"" + std::string(kKnobNames[k]) + ":" + std::to_string(b) + "\": " + std::to_string(c);
    }
  return out + "}";
}

void tune_from_json(const std::string& js) {
  // {"name:bucket": int, ...}; whitespace anywhere between tokens
  int table[kTuneKnobs][kTuneBuckets];
  for (auto& row : table)
    for (int& c : row) c = -1;
  size_t i = 0;
  auto skip = [&] {
    while (i < js.size() && std::isspace((unsigned char)js[i])) i++;
  };
  auto bad = [](const char* what) { throw std::invalid_argument(std::string("tune json: ") + what); };
  skip();
  if (i >= js.size() || js[i] != '{') bad("expected '{'");
  i++;
  skip();
  if (i < js.size() && js[i] == '}') {
    i++;
  } else {
    for (;;) {
      skip();
      if (i >= js.size() || js[i] != '"') bad("expected a key");
      const size_t e = js.find('"', i + 1);
      if (e == std::string::npos) bad("unterminated key");
      const std::string key = js.substr(i + 1, e - i - 1);
      i = e + 1;
      skip();
      if (i >= js.size() || js[i] != ':') bad("expected ':'");
      i++;
      skip();
      size_t j = i;
      if (j < js.size() && js[j] == '-') j++;
      while (j < js.size() && std::isdigit((unsigned char)js[j])) j++;
      if (j == i) bad("expected an integer");
      const int val = std::atoi(js.substr(i, j - i).c_str());
      i = j;
      int knob = -1, bucket = -1;
      if (!tune_parse_stage("tune:" + key, &knob, &bucket)) bad("unknown knob");
      if (bucket < 0 || bucket >= kTuneBuckets) bad("bucket out of range");
      if (val < -1 || val >= kTuneCandidates[knob]) bad("candidate out of range");
      table[knob][bucket] = val;
      skip();
      if (i < js.size() && js[i] == ',') {
        i++;
        continue;
      }
      if (i < js.size() && js[i] == '}') {
        i++;
        break;
      }
      bad("expected ',' or '}'");
    }
  }
  skip();
  if (i != js.size()) bad("trailing characters");
  for (int k = 0; k < kTuneKnobs; k++)
    for (int b = 0; b < kTuneBuckets; b++) g_table[k][b].store(table[k][b]);
}

}  // namespace ki
