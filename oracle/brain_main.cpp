// Test infrastructure only: the `brain -anatomy HGG_UQ` entry of
// source/Glioma/Glioma_main.cpp:46-104 reduced to the one driver on the hot
// path, so the reference's own Glioma_HG_UQ.cpp can be linked without the
// out-of-scope drivers that Glioma_main.cpp also pulls in.
#include "Glioma_HG_UQ.h"
int main(int argc, const char **argv) {
    ArgumentParser parser(argc, argv);
    Environment::setup(std::max(1, parser("-nthreads").asInt()));
    Glioma *s = new Glioma_HG_UQ(argc, argv);
    s->run();
    delete s;
    return 0;
}
