// Stand-in for pwm's include/wx_base.hpp (test infrastructure only): the
// static traits every registered construction inherits.
#pragma once
template <bool external_in_, bool external_out_, bool stats_support_ = false, bool is_inplace_ = false>
class wx_in_out_external {
 public:
  static constexpr bool external_in = external_in_;
  static constexpr bool external_out = external_out_;
  static constexpr bool stats_support = stats_support_;
  static constexpr bool is_inplace = is_inplace_;
};
