// main() of the GoogleTest stand-in (gtest/gtest.h): runs every registered
// test, or those whose "Suite.Name" contains the text of --gtest_filter=.
#include <gtest/gtest.h>

int main(int argc, char** argv) {
    std::string filter;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a.rfind("--gtest_filter=", 0) == 0) filter = a.substr(15);
    }
    return ::testing::internal::run_all(filter) == 0 ? 0 : 1;
}
