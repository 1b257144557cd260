// Minimal stand-in for the GoogleTest macros used by the lbm-2d unit tests
// (TEST, EXPECT_*), so those tests build without fetching GoogleTest.
// LBM2D_TEST_FILTER=substring runs only the tests whose "Suite.Name"
// contains the substring; LBM2D_TEST_SKIP=substring skips matching tests.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <string>
#include <vector>

namespace shim {
struct Case {
    std::string name;
    std::function<void()> fn;
};
inline std::vector<Case>& registry() {
    static std::vector<Case> r;
    return r;
}
inline int& failures() {
    static int f = 0;
    return f;
}
struct Reg {
    Reg(const char* suite, const char* name, std::function<void()> fn) {
        registry().push_back({std::string(suite) + "." + name, std::move(fn)});
    }
};
inline void fail(const char* file, int line, const std::string& what) {
    std::printf("  FAILED %s:%d: %s\n", file, line, what.c_str());
    ++failures();
}
}  // namespace shim

#define TEST(suite, name)                                                          \
    static void suite##_##name##_body();                                           \
    static shim::Reg suite##_##name##_reg(#suite, #name, suite##_##name##_body);   \
    static void suite##_##name##_body()

#define SHIM_CHECK(cond, text) \
    do {                       \
        if (!(cond)) shim::fail(__FILE__, __LINE__, text); \
    } while (0)
#define EXPECT_TRUE(c) SHIM_CHECK((c), #c)
#define EXPECT_FALSE(c) SHIM_CHECK(!(c), "!(" #c ")")
#define EXPECT_EQ(a, b) SHIM_CHECK((a) == (b), #a " == " #b)
#define EXPECT_NE(a, b) SHIM_CHECK((a) != (b), #a " != " #b)
#define EXPECT_GT(a, b) SHIM_CHECK((a) > (b), #a " > " #b)
#define EXPECT_LT(a, b) SHIM_CHECK((a) < (b), #a " < " #b)
#define EXPECT_GE(a, b) SHIM_CHECK((a) >= (b), #a " >= " #b)
#define EXPECT_LE(a, b) SHIM_CHECK((a) <= (b), #a " <= " #b)
#define EXPECT_NEAR(a, b, tol) SHIM_CHECK(std::fabs((double)(a) - (double)(b)) <= (tol), #a " ~ " #b)
#define EXPECT_DOUBLE_EQ(a, b) \
    SHIM_CHECK(std::fabs((double)(a) - (double)(b)) <= 4 * 2.220446049250313e-16 * std::fabs((double)(b)) + 1e-300, \
               #a " == " #b)
#define ASSERT_TRUE EXPECT_TRUE
#define ASSERT_EQ EXPECT_EQ
#define ASSERT_NEAR EXPECT_NEAR

int main() {
    const char* only = std::getenv("LBM2D_TEST_FILTER");
    const char* skip = std::getenv("LBM2D_TEST_SKIP");
    int run = 0, bad = 0;
    for (auto& c : shim::registry()) {
        if (only && c.name.find(only) == std::string::npos) continue;
        if (skip && *skip && c.name.find(skip) != std::string::npos) continue;
        const int before = shim::failures();
        try {
            c.fn();
        } catch (const std::exception& e) {
            shim::fail(__FILE__, __LINE__, std::string("exception: ") + e.what());
        }
        ++run;
        const bool ok = shim::failures() == before;
        if (!ok) ++bad;
        std::printf("[%s] %s\n", ok ? "  OK  " : " FAIL ", c.name.c_str());
    }
    std::printf("%d tests, %d failed\n", run, bad);
    return bad ? 1 : 0;
}
