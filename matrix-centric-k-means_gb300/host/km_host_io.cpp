// C entry points of km_host.h over InputParser (input_parser.hpp).
#include "km_host.h"

#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "input_parser.hpp"

namespace {

using Parser = InputParser<float>;

int copy_out(Parser& p, uint32_t d, uint64_t n, float* out, uint64_t* rows_read) {
  std::memcpy(out, p.data(), sizeof(float) * d * n);
  if (rows_read) *rows_read = p.rows_read();
  return 0;
}

}  // namespace

extern "C" {

int kmh_parse_points(const char* text, uint64_t len, int32_t svm, uint32_t d, uint64_t n,
                     int32_t csv_plain, float* out, uint64_t* rows_read) {
  if (!text || !out || d == 0 || n == 0) return 1;
  std::istringstream in(std::string(text, len));
  Parser::InputFormat f = svm ? Parser::InputFormat::SVM : Parser::InputFormat::CSV;
  Parser p(in, static_cast<int>(d), n, f, csv_plain ? Parser::CsvColumns::plain : Parser::CsvColumns::reference);
  return copy_out(p, d, n, out, rows_read);
}

int kmh_read_points(const char* path, uint32_t d, uint64_t n, int32_t csv_plain, float* out,
                    uint64_t* rows_read) {
  if (!path || !out || d == 0 || n == 0) return 1;
  const std::string name(path);
  Parser::InputFormat f;
  if (name.find(".csv") != std::string::npos) f = Parser::InputFormat::CSV;
  else if (name.find(".svm") != std::string::npos) f = Parser::InputFormat::SVM;
  else return 4;
  std::ifstream in(name, std::ios::in | std::ios::binary);
  if (!in) return 4;
  Parser p(in, static_cast<int>(d), n, f, csv_plain ? Parser::CsvColumns::plain : Parser::CsvColumns::reference);
  return copy_out(p, d, n, out, rows_read);
}

int kmh_random_points(int32_t seed, uint32_t d, uint64_t n, float* out) {
  if (!out || d == 0 || n == 0) return 1;
  Parser p(seed, static_cast<int>(d), n);
  std::memcpy(out, p.data(), sizeof(float) * d * n);
  return 0;
}

int kmh_write_csv(const char* path, const float* X, const uint32_t* labels, uint32_t d, uint64_t n) {
  if (!path || !X || !labels || d == 0 || n == 0) return 1;
  Parser p(X, static_cast<int>(d), n);
  std::memcpy(p.clusters(), labels, sizeof(uint32_t) * n);
  std::ofstream o(path, std::ios::out | std::ios::binary);
  if (!o) return 4;
  p.dataset_to_csv(o);
  return o ? 0 : 4;
}

}  // extern "C"
