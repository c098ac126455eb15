// cadise-gb300: render CRSD scene files on the GPU (the reference's CLI takes
// each argument as a scene file, source/file-io/clParser.cpp:13-34).
// Writes <output-filename stem>.ppm (sRGB) and .pfm (linear) per scene.
#include "cadise_host.h"

#include <cstdio>
#include <string>

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s scene.crsd [scene.crsd ...]\n", argv[0]);
        return 2;
    }
    int rc = 0;
    for (int i = 1; i < argc; ++i) {
        try {
            cadise_gb300::RenderSession s(argv[i]);
            s.render();
            std::string out = s.scene()->settings().output_filename;
            const size_t dot = out.find_last_of('.');
            if (dot != std::string::npos) out = out.substr(0, dot);
            s.save(out);
            std::printf("%s: %dx%d, %d spp, %.1f ms -> %s.ppm / %s.pfm\n", argv[i], s.film().width(), s.film().height(),
                        s.scene()->settings().spp, s.renderMs(), out.c_str(), out.c_str());
        } catch (const cadise_gb300::Error& e) {
            std::fprintf(stderr, "%s: %s\n", argv[i], e.what());
            rc = 1;
        }
    }
    return rc;
}
