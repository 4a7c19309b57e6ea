/*
 * km_host.h — C entry points of libkmeans_host (host C++, no device code):
 * the gpukmeans dataset reader and writer (input_parser.hpp) for callers that
 * are not C++, e.g. ctypes.
 *
 * Reference interfaces replaced:
 *   InputParser(istream&, d, n, format)   src/include/input_parser.hpp:28-46, :76-131
 *   InputParser(seed, d, n)               src/include/input_parser.hpp:50-68
 *   InputParser::dataset_to_csv(ostream&) src/include/input_parser.hpp:167-183
 */
#ifndef KM_HOST_H
#define KM_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reads n points of d coordinates from `path` (".csv" or ".svm" in the name
 * selects the format, as gpukmeans does) into out (n*d floats, row-major).
 * csv_plain == 0 drops CSV column 0 (the reference's reader), 1 keeps it.
 * rows_read receives the data rows found (at most n).  Returns 0 on success,
 * 4 when the file cannot be opened or has another suffix (the reference's
 * EXIT_INVALID_INFILE), 1 on a bad argument. */
int kmh_read_points(const char* path, uint32_t d, uint64_t n, int32_t csv_plain, float* out,
                    uint64_t* rows_read);

/* The same on an in-memory text (svm != 0: libsvm, else CSV). */
int kmh_parse_points(const char* text, uint64_t len, int32_t svm, uint32_t d, uint64_t n,
                     int32_t csv_plain, float* out, uint64_t* rows_read);

/* The reference's seeded random points: mt19937(seed),
 * uniform_real_distribution<float>(-1e5, 1e5), row-major. */
int kmh_random_points(int32_t seed, uint32_t d, uint64_t n, float* out);

/* Writes the reference's output CSV (header "cluster,d0,...", rows
 * "label,values" with 8 significant digits) of n points to `path`. */
int kmh_write_csv(const char* path, const float* X, const uint32_t* labels, uint32_t d, uint64_t n);

#ifdef __cplusplus
}
#endif

#endif /* KM_HOST_H */
