// A small stand-in for the part of GoogleTest that MDcraft's C++ tests use
// (test/cxx/**/*.cxx): TEST, TEST_F over a testing::Test fixture, the
// EXPECT_/ASSERT_ comparison macros with streamed messages, EXPECT_THROW,
// and a runner (main() in gtest_main.cpp beside this header) that runs
// every registered test and prints a summary. It lets those test sources
// compile, unmodified, against this library's drop-in headers where
// GoogleTest itself is not installed. A failure prints the file, line and
// values; the ASSERT_ forms return from the test body.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <exception>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace testing {

class Test {
public:
    virtual ~Test() = default;
    virtual void SetUp() {}
    virtual void TearDown() {}
    virtual void TestBody() = 0;
};

namespace internal {

struct Registered {
    std::string suite, name;
    std::function<Test*()> make;
};

inline std::vector<Registered>& registry() {
    static std::vector<Registered> r;
    return r;
}

inline int& current_failures() {
    static int n = 0;
    return n;
}

struct Registrar {
    Registrar(const char* suite, const char* name, std::function<Test*()> make) {
        registry().push_back({suite, name, std::move(make)});
    }
};

// Collects a failure's message (the check's own text plus anything the test
// streams into it) and prints it when the statement ends.
class Failure {
public:
    Failure(const char* file, int line, const std::string& what) {
        ss_ << file << ":" << line << ": Failure\n" << what;
        ++current_failures();
    }
    Failure(const Failure& o) : ss_(o.ss_.str()) {}
    ~Failure() {
        if (!ss_.str().empty()) std::cout << ss_.str() << "\n" << std::flush;
    }
    template <class T>
    Failure& operator<<(const T& v) {
        ss_ << v;
        return *this;
    }
    void clear() { ss_.str(""); }

private:
    std::ostringstream ss_;
};

// Absorbs the streamed message of a check that passed.
struct Passed {
    template <class T>
    Passed& operator<<(const T&) {
        return *this;
    }
};

// Lets `return Assign() = Failure(...) << msg;` end a void test body.
struct ReturnVoid {
    void operator=(const Failure&) const {}
};

template <class T>
std::string show(const T& v) {
    std::ostringstream s;
    s << v;
    return s.str();
}
inline std::string show(bool v) { return v ? "true" : "false"; }
inline std::string show(std::nullptr_t) { return "nullptr"; }

template <class A, class B>
std::string cmp_text(const char* op, const char* ea, const char* eb, const A& a, const B& b) {
    std::ostringstream s;
    s << "Expected: (" << ea << ") " << op << " (" << eb << "), actual: " << show(a) << " vs " << show(b) << "\n";
    return s.str();
}

// EXPECT_DOUBLE_EQ's test: within 4 units in the last place, NaN never equal.
inline bool almost_equal(double a, double b) {
    if (std::isnan(a) || std::isnan(b)) return false;
    if (a == b) return true;
    auto biased = [](double x) {
        unsigned long long u;
        std::memcpy(&u, &x, sizeof(u));
        const unsigned long long sign = 1ull << 63;
        return (u & sign) ? ~u + 1 : u | sign;
    };
    const unsigned long long ua = biased(a), ub = biased(b);
    return (ua > ub ? ua - ub : ub - ua) <= 4;
}

// Runs every registered test whose "Suite.Name" contains `filter` (all when
// it is empty); returns the number of failed tests.
inline int run_all(const std::string& filter) {
    int failed = 0, ran = 0;
    for (const Registered& r : registry()) {
        const std::string full = r.suite + "." + r.name;
        if (!filter.empty() && full.find(filter) == std::string::npos) continue;
        ++ran;
        std::cout << "[ RUN      ] " << full << "\n" << std::flush;
        current_failures() = 0;
        Test* t = nullptr;
        try {
            t = r.make();
            t->SetUp();
            t->TestBody();
            t->TearDown();
        } catch (const std::exception& e) {
            std::cout << "uncaught exception: " << e.what() << "\n";
            ++current_failures();
        } catch (...) {
            std::cout << "uncaught exception\n";
            ++current_failures();
        }
        delete t;
        const bool ok = current_failures() == 0;
        failed += ok ? 0 : 1;
        std::cout << (ok ? "[       OK ] " : "[  FAILED  ] ") << full << "\n" << std::flush;
    }
    std::cout << "[==========] " << ran << " tests ran, " << failed << " failed\n";
    return failed;
}

}  // namespace internal
}  // namespace testing

#define MDG_GT_CLASS(suite, name) suite##_##name##_Test

#define TEST(suite, name)                                                                                \
    class MDG_GT_CLASS(suite, name) : public ::testing::Test {                                           \
    public:                                                                                              \
        void TestBody() override;                                                                        \
    };                                                                                                   \
    static ::testing::internal::Registrar mdg_gt_reg_##suite##_##name(                                   \
        #suite, #name, [] { return static_cast<::testing::Test*>(new MDG_GT_CLASS(suite, name)); });    \
    void MDG_GT_CLASS(suite, name)::TestBody()

#define TEST_F(fixture, name)                                                                            \
    class MDG_GT_CLASS(fixture, name) : public fixture {                                                 \
    public:                                                                                              \
        void TestBody() override;                                                                        \
    };                                                                                                   \
    static ::testing::internal::Registrar mdg_gt_reg_##fixture##_##name(                                 \
        #fixture, #name, [] { return static_cast<::testing::Test*>(new MDG_GT_CLASS(fixture, name)); }); \
    void MDG_GT_CLASS(fixture, name)::TestBody()

// A passing check swallows the streamed message; a failing one prints it.
#define MDG_GT_CHECK(cond, text)                                                                         \
    if (cond)                                                                                            \
        ::testing::internal::Passed();                                                                   \
    else                                                                                                 \
        ::testing::internal::Failure(__FILE__, __LINE__, text)

#define MDG_GT_ASSERT(cond, text)                                                                        \
    if (cond) {                                                                                          \
    } else                                                                                               \
        return ::testing::internal::ReturnVoid() = ::testing::internal::Failure(__FILE__, __LINE__, text)

#define MDG_GT_BIN(kind, op, a, b) kind(((a)op(b)), ::testing::internal::cmp_text(#op, #a, #b, (a), (b)))

#define EXPECT_EQ(a, b) MDG_GT_BIN(MDG_GT_CHECK, ==, a, b)
#define EXPECT_NE(a, b) MDG_GT_BIN(MDG_GT_CHECK, !=, a, b)
#define EXPECT_LT(a, b) MDG_GT_BIN(MDG_GT_CHECK, <, a, b)
#define EXPECT_LE(a, b) MDG_GT_BIN(MDG_GT_CHECK, <=, a, b)
#define EXPECT_GT(a, b) MDG_GT_BIN(MDG_GT_CHECK, >, a, b)
#define EXPECT_GE(a, b) MDG_GT_BIN(MDG_GT_CHECK, >=, a, b)
#define ASSERT_EQ(a, b) MDG_GT_BIN(MDG_GT_ASSERT, ==, a, b)
#define ASSERT_NE(a, b) MDG_GT_BIN(MDG_GT_ASSERT, !=, a, b)
#define ASSERT_LT(a, b) MDG_GT_BIN(MDG_GT_ASSERT, <, a, b)
#define ASSERT_LE(a, b) MDG_GT_BIN(MDG_GT_ASSERT, <=, a, b)
#define ASSERT_GT(a, b) MDG_GT_BIN(MDG_GT_ASSERT, >, a, b)
#define ASSERT_GE(a, b) MDG_GT_BIN(MDG_GT_ASSERT, >=, a, b)
#define EXPECT_TRUE(c) MDG_GT_CHECK(static_cast<bool>(c), std::string("Expected true: " #c "\n"))
#define EXPECT_FALSE(c) MDG_GT_CHECK(!static_cast<bool>(c), std::string("Expected false: " #c "\n"))
#define ASSERT_TRUE(c) MDG_GT_ASSERT(static_cast<bool>(c), std::string("Expected true: " #c "\n"))
#define ASSERT_FALSE(c) MDG_GT_ASSERT(!static_cast<bool>(c), std::string("Expected false: " #c "\n"))
#define EXPECT_NEAR(a, b, tol)                                                                           \
    MDG_GT_CHECK(std::fabs(double(a) - double(b)) <= double(tol),                                        \
                 ::testing::internal::cmp_text("within " #tol " of", #a, #b, (a), (b)))
#define ASSERT_NEAR(a, b, tol)                                                                           \
    MDG_GT_ASSERT(std::fabs(double(a) - double(b)) <= double(tol),                                       \
                  ::testing::internal::cmp_text("within " #tol " of", #a, #b, (a), (b)))
#define EXPECT_DOUBLE_EQ(a, b)                                                                           \
    MDG_GT_CHECK(::testing::internal::almost_equal(double(a), double(b)),                               \
                 ::testing::internal::cmp_text("~==", #a, #b, (a), (b)))
#define ASSERT_DOUBLE_EQ(a, b)                                                                           \
    MDG_GT_ASSERT(::testing::internal::almost_equal(double(a), double(b)),                              \
                  ::testing::internal::cmp_text("~==", #a, #b, (a), (b)))
#define EXPECT_THROW(stmt, exc)                                                                          \
    MDG_GT_CHECK(([&]() -> bool {                                                                        \
                     try {                                                                               \
                         stmt;                                                                           \
                     } catch (const exc&) {                                                              \
                         return true;                                                                    \
                     } catch (...) {                                                                     \
                     }                                                                                   \
                     return false;                                                                       \
                 }()),                                                                                   \
                 std::string("Expected " #stmt " to throw " #exc "\n"))
