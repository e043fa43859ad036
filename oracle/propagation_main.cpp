// Test infrastructure only: the `-anatomy HGG_Propagation` entry of
// source/Glioma/Glioma_main.cpp reduced to that one driver, so the reference's
// own Glioma_HG_Propagation.cpp (posterior mean and variance fields over the
// samples' HGG_data.dat files) links without the other drivers.
#include "Glioma_HG_Propagation.h"
int main(int argc, const char **argv) {
    ArgumentParser parser(argc, argv);
    Environment::setup(std::max(1, parser("-nthreads").asInt()));
    Glioma *s = new Glioma_HG_Propagation(argc, argv);
    s->run();
    delete s;
    return 0;
}
