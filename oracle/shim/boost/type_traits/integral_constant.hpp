// Empty: pagmo includes this header but uses std::integral_constant.
