// Result sinks: human-readable stdout or an appending CSV file.
//
// Same observable formats as sycl-bench's include/result_consumer.h:
//   stdout (:29-51):  "********** Results for <name>**********" then
//                     "<result>: <value>[ [<unit>]]" per line
//   CSV    (:54-106): at every flush, a header "# Benchmark name,<columns>"
//                     with the columns sorted by std::sort, then one row per
//                     buffered benchmark; units are dropped.
#pragma once

#include <algorithm>
#include <cassert>
#include <fstream>
#include <map>
#include <ostream>
#include <set>
#include <string>
#include <vector>

class ResultConsumer {
public:
  virtual void proceedToBenchmark(const std::string& name) = 0;
  virtual void consumeResult(const std::string& result_name, const std::string& result,
      const std::string& unit = "") = 0;
  // Guarantees the results have been written out.
  virtual void flush() = 0;
  // Drops the current benchmark's results (after an error).
  virtual void discard() {}
  virtual ~ResultConsumer() = default;
};

class OstreamResultConsumer : public ResultConsumer {
public:
  explicit OstreamResultConsumer(std::ostream& out) : out_(out) {}

  void proceedToBenchmark(const std::string& name) override {
    out_ << "********** Results for " << name << "**********" << std::endl;
  }

  void consumeResult(const std::string& result_name, const std::string& result, const std::string& unit = "") override {
    out_ << result_name << ": " << result;
    if(!unit.empty()) out_ << " [" << unit << "]";
    out_ << std::endl;
  }

  void flush() override {}

private:
  std::ostream& out_;
};

class AppendingCsvResultConsumer : public ResultConsumer {
public:
  explicit AppendingCsvResultConsumer(const std::string& path) : file_(path, std::ios::app) {}

  void proceedToBenchmark(const std::string& name) override { current_ = name; }

  void consumeResult(const std::string& result_name, const std::string& result, const std::string& = "") override {
    rows_[current_][result_name] = result;
  }

  void flush() override {
    std::set<std::string> unique;
    for(const auto& row : rows_)
      for(const auto& cell : row.second) unique.insert(cell.first);
    std::vector<std::string> columns(unique.begin(), unique.end());
    std::sort(columns.begin(), columns.end());

    file_ << "# Benchmark name";
    for(const auto& c : columns) file_ << "," << c;
    file_ << std::endl;
    for(const auto& row : rows_) {
      file_ << row.first;
      for(const auto& c : columns) {
        auto it = row.second.find(c);
        // every row of one flush carries the same columns; a missing cell would
        // be a harness bug (the reference throws from map::at here)
        if(it == row.second.end()) throw std::out_of_range("missing CSV cell " + c);
        file_ << "," << it->second;
      }
      file_ << std::endl;
    }
    rows_.clear();
  }

  void discard() override {
    assert(!current_.empty());
    rows_.erase(current_);
    current_.clear();
  }

private:
  std::string current_;
  std::map<std::string, std::map<std::string, std::string>> rows_;
  std::ofstream file_;
};
