// Walks an HDF5 file with the map reader's own structures (h5_map.cpp is
// compiled into this program): the superblock, the root group's links and,
// for every link, the dataset the reader describes.  One line per link:
//
//   link <name> class <c> elem <bytes> order <le|be> dims <d0,d1,...> address <absolute>
//   link <name> error <code> <message>
//
// then the result of the map entry point on the same file:
//
//   map <status> <chunks> <edge> <error message>
//
// Exit status 0 unless the superblock or the root group cannot be read.
#include "h5_map.cpp"

#include <cstdarg>
#include <cstdio>
#include <cstdlib>

namespace tsdfl {
static char g_error[512];
void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_error, sizeof(g_error), fmt, ap);
    va_end(ap);
}
}  // namespace tsdfl

int main(int argc, char** argv)
{
    using namespace tsdfl;
    if (argc != 2) {
        std::fprintf(stderr, "usage: h5_walk FILE\n");
        return 2;
    }
    try {
        H5File f(argv[1]);
        std::printf("superblock offsets %d lengths %d root %llu\n", f.so(), f.sl(), (unsigned long long)f.root());
        for (const auto& l : f.links(f.root())) {
            try {
                const DatasetInfo d = f.describe(l.second);
                std::printf("link %s class %d elem %u order %s dims ", l.first.c_str(), d.type_class, d.elem,
                            d.big_endian ? "be" : "le");
                for (size_t i = 0; i < d.dims.size(); ++i)
                    std::printf("%s%llu", i ? "," : "", (unsigned long long)d.dims[i]);
                std::printf(" address %llu\n", (unsigned long long)d.address);
            } catch (const H5Error& e) {
                std::printf("link %s error %d %s\n", l.first.c_str(), e.code, e.msg.c_str());
            }
        }
    } catch (const H5Error& e) {
        std::printf("error %d %s\n", e.code, e.msg.c_str());
        return 1;
    }
    int32_t* pos = nullptr;
    uint32_t* raw = nullptr;
    size_t n = 0;
    int32_t edge = 0;
    g_error[0] = 0;
    const int rc = tsdfl_read_map_h5(argv[1], &pos, &raw, &n, &edge);
    std::printf("map %d %zu %d %s\n", rc, n, edge, g_error);
    std::free(pos);
    std::free(raw);
    return 0;
}
