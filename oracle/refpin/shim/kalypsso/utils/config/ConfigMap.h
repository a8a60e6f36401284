// Key/value parameters (stand-in for the kalypsso ConfigMap read from an ini file).
#pragma once
#include <map>
#include <string>
#include <cstdlib>
#include <vector>
namespace kalypsso
{
class ConfigMap
{
public:
  std::map<std::string, std::string> kv;
  void set(const std::string & s, const std::string & k, const std::string & v) { kv[s + "/" + k] = v; }
  std::string getString(const std::string & s, const std::string & k, const std::string & d) const
  {
    auto it = kv.find(s + "/" + k);
    return it == kv.end() ? d : it->second;
  }
  double getReal(const std::string & s, const std::string & k, double d) const
  {
    auto it = kv.find(s + "/" + k);
    return it == kv.end() ? d : std::strtod(it->second.c_str(), nullptr);
  }
  int getInteger(const std::string & s, const std::string & k, int d) const
  {
    auto it = kv.find(s + "/" + k);
    return it == kv.end() ? d : std::atoi(it->second.c_str());
  }
  std::vector<double> getRealVector(const std::string &, const std::string &, std::vector<double> d) const { return d; }
  bool getBool(const std::string & s, const std::string & k, bool d) const
  {
    auto it = kv.find(s + "/" + k);
    return it == kv.end() ? d : (it->second == "yes" || it->second == "true" || it->second == "1");
  }
};
} // namespace kalypsso
using kalypsso::ConfigMap;
