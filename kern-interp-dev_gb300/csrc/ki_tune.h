// Launch choices per box-size bucket, picked by the library's autotuner
// (ki_autotune): for each tunable launch group of the factorization and the
// solve, the candidate shape that ran fastest for that bucket on this GPU.
// A bucket the table does not name takes the built-in heuristic.
#pragma once

#include <string>

namespace ki {

enum TuneKnob : int {
  // k_id bins.  FP32: 0 {32 fold rows, 256 threads}, 1 {64, 256},
  // 2 {32, 512}, 3 {64, 512}; FP64: 0 {32, 256}, 1 {64, 256}.  Bucket: the
  // bin's group and largest n (id_bucket).  A 64-row fold that does not fit
  // in shared memory falls back to 32.
  kTuneId = 0,
  // k_schur shared-memory bins.  FP32: threads 256, 512, 1024 for
  // candidates 0-2 with the Gauss-Jordan split where the bin allows it,
  // 3-5 the same without the split; FP64: 128 or 256 threads.  Bucket: the
  // bin's largest redundant block and CTAs per SM (schur_bucket).
  kTuneSchur = 1,
  // k_sweep launches: 128, 256 or 512 threads.  Bucket: the level's largest
  // active set (sweep_bucket).
  kTuneSweep = 2,
  kTuneKnobs = 3
};

constexpr int kTuneBuckets = 512;
constexpr int kTuneCandidates[kTuneKnobs] = {4, 6, 3};

// Buckets; the precision is part of the key (FP64 in the upper half).
int id_bucket(bool fp64, int group, int n_max);
int schur_bucket(bool fp64, int r_max, int per_sm);
int sweep_bucket(bool fp64, int n_max);

// The candidate for (knob, bucket): the forced one while the tuner measures
// a candidate, else the table's, else -1 (the built-in heuristic).
int tune_choice(int knob, int bucket);
void tune_set(int knob, int bucket, int choice);
void tune_clear();
// Force one candidate on every bucket of a knob (-1: back to the table).
void tune_force(int knob, int choice);
// While on, the factorization and the solve bracket every tunable launch
// with events named tune_stage(knob, bucket) and run on one stream.
bool tune_recording();
void tune_set_recording(bool on);
std::string tune_stage(int knob, int bucket);
// Parses a tune_stage name; false for other stage names.
bool tune_parse_stage(const std::string& s, int* knob, int* bucket);

// The table as a flat JSON object {"id:17": 2, ...} and back; tune_from_json
// replaces the table and throws std::invalid_argument on malformed input.
std::string tune_to_json();
void tune_from_json(const std::string& json);

}  // namespace ki
