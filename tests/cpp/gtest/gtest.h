// Minimal GoogleTest-compatible harness (test infrastructure): enough of the macro set
// for the reference's unit tests to compile unchanged against this library's headers.
#pragma once
#include <cmath>
#include <cstdio>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace testing {
struct Registry {
    struct Case { std::string name; std::function<void()> fn; };
    static std::vector<Case> &cases() { static std::vector<Case> c; return c; }
    static int &failures() { static int f = 0; return f; }
};
struct Registrar {
    Registrar(const char *suite, const char *name, std::function<void()> fn) {
        Registry::cases().push_back({std::string(suite) + "." + name, std::move(fn)});
    }
};
struct AssertFail {};
inline void InitGoogleTest(int *, char **) {}
inline void report(const char *file, int line, const std::string &what) {
    ++Registry::failures();
    std::cerr << file << ":" << line << ": Failure: " << what << std::endl;
}
}  // namespace testing

inline int RUN_ALL_TESTS() {
    int failedCases = 0;
    for (auto &c : testing::Registry::cases()) {
        const int before = testing::Registry::failures();
        try { c.fn(); } catch (testing::AssertFail &) {
        } catch (std::exception &e) {
            testing::report(__FILE__, __LINE__, std::string("uncaught exception: ") + e.what());
        }
        const bool ok = testing::Registry::failures() == before;
        std::cout << (ok ? "[       OK ] " : "[  FAILED  ] ") << c.name << std::endl;
        failedCases += ok ? 0 : 1;
    }
    std::cout << testing::Registry::cases().size() - failedCases << " passed, " << failedCases << " failed" << std::endl;
    return failedCases == 0 ? 0 : 1;
}

#define EIKX_GT_CAT(a, b) a##b
#define TEST(suite, name)                                                                      \
    static void EIKX_GT_CAT(suite##_, name)();                                                 \
    static testing::Registrar EIKX_GT_CAT(reg_##suite##_, name)(#suite, #name,                 \
                                                                 EIKX_GT_CAT(suite##_, name)); \
    static void EIKX_GT_CAT(suite##_, name)()

#define EIKX_GT_CHECK(cond, text, fatal)                                                       \
    do {                                                                                       \
        if (!(cond)) {                                                                         \
            testing::report(__FILE__, __LINE__, text);                                          \
            if (fatal) throw testing::AssertFail{};                                            \
        }                                                                                      \
    } while (0)
#define EXPECT_TRUE(c) EIKX_GT_CHECK((c), #c, false)
#define EXPECT_FALSE(c) EIKX_GT_CHECK(!(c), "!(" #c ")", false)
#define ASSERT_TRUE(c) EIKX_GT_CHECK((c), #c, true)
#define ASSERT_FALSE(c) EIKX_GT_CHECK(!(c), "!(" #c ")", true)
#define EXPECT_EQ(a, b) EIKX_GT_CHECK(((a) == (b)), #a " == " #b, false)
#define EXPECT_NE(a, b) EIKX_GT_CHECK(((a) != (b)), #a " != " #b, false)
#define EXPECT_LT(a, b) EIKX_GT_CHECK(((a) < (b)), #a " < " #b, false)
#define EXPECT_LE(a, b) EIKX_GT_CHECK(((a) <= (b)), #a " <= " #b, false)
#define EXPECT_GT(a, b) EIKX_GT_CHECK(((a) > (b)), #a " > " #b, false)
#define EXPECT_GE(a, b) EIKX_GT_CHECK(((a) >= (b)), #a " >= " #b, false)
#define ASSERT_EQ(a, b) EIKX_GT_CHECK(((a) == (b)), #a " == " #b, true)
#define ASSERT_NE(a, b) EIKX_GT_CHECK(((a) != (b)), #a " != " #b, true)
#define EXPECT_NEAR(a, b, tol) EIKX_GT_CHECK((std::abs(static_cast<double>(a) - static_cast<double>(b)) <= (tol)), \
                                             #a " ~ " #b, false)
#define ASSERT_NEAR(a, b, tol) EIKX_GT_CHECK((std::abs(static_cast<double>(a) - static_cast<double>(b)) <= (tol)), \
                                             #a " ~ " #b, true)
#define EXPECT_NO_THROW(stmt)                                                                  \
    do {                                                                                       \
        try { stmt; } catch (std::exception &e_) {                                             \
            testing::report(__FILE__, __LINE__, std::string(#stmt " threw: ") + e_.what());    \
        }                                                                                      \
    } while (0)
#define ASSERT_NO_THROW(stmt) EXPECT_NO_THROW(stmt)
#define EXPECT_THROW(stmt, exc)                                                                \
    do {                                                                                       \
        bool thrown_ = false;                                                                  \
        try { stmt; } catch (exc &) { thrown_ = true; } catch (...) {}                          \
        EIKX_GT_CHECK(thrown_, #stmt " did not throw " #exc, false);                           \
    } while (0)
#define EXPECT_ANY_THROW(stmt)                                                                 \
    do {                                                                                       \
        bool thrown_ = false;                                                                  \
        try { stmt; } catch (...) { thrown_ = true; }                                           \
        EIKX_GT_CHECK(thrown_, #stmt " did not throw", false);                                 \
    } while (0)
