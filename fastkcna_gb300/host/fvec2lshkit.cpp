// fvec2lshkit - converts a .fvecs file (per vector: int32 d, then d float32)
// into the lshkit layout the build tools read (u32 header {4, n, d}, then the
// n x d floats row-major), as src/fvec2lshit.cpp does.
//
// Same command line, output bytes and console lines as the reference tool:
//   fvec2lshkit <input> <output>     (any other argument count prints this
//                                     usage line and exits 0)
// prints "dim:  d", "n:  n" and the first vector.  n is the file size over the
// record size 4 + 4d; a trailing partial record is ignored.  The records are
// streamed through one buffer of whole records (64 MiB) instead of one
// read per vector.  Errors: the reference aborts through BOOST_VERIFY when a
// record's length field differs from d (and reads garbage from an unreadable
// input); here every such case prints a message on stderr and exits 1, and the
// output is left incomplete.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

namespace {

int fail(const std::string &msg) {
    std::cerr << "fvec2lshkit: " << msg << std::endl;
    return 1;
}

} // namespace

int main(int argc, char *argv[]) {
    if (argc != 3) {
        std::cout << "fvec2lshkit <input> <output>" << std::endl;
        return 0;
    }
    std::ifstream is(argv[1], std::ios::binary);
    if (!is) return fail(std::string("cannot open ") + argv[1]);
    std::ofstream os(argv[2], std::ios::binary);
    if (!os) return fail(std::string("cannot create ") + argv[2]);

    int32_t d = 0;
    if (!is.read(reinterpret_cast<char *>(&d), 4)) return fail("input shorter than one length field");
    std::cout << "dim:  " << d << std::endl;
    if (d <= 0) return fail("non-positive dimension " + std::to_string(d));
    is.seekg(0, std::ios::end);
    const uint64_t bytes = (uint64_t)is.tellg();
    const uint64_t rec = 4 + 4 * (uint64_t)d;
    const uint64_t n64 = bytes / rec;
    if (n64 > 0xFFFFFFFFull) return fail("more than 2^32 - 1 vectors");
    const int32_t n = (int32_t)n64;
    std::cout << "n:  " << n << std::endl;
    const int32_t header[3] = {4, n, d};
    os.write(reinterpret_cast<const char *>(header), sizeof header);
    is.seekg(0, std::ios::beg);

    const uint64_t per = std::max<uint64_t>(1, (64ull << 20) / rec); // records per chunk
    std::vector<char> in((size_t)(per * rec));
    std::vector<float> out((size_t)(per * (uint64_t)d));
    for (uint64_t i0 = 0; i0 < n64; i0 += per) {
        const uint64_t m = std::min(per, n64 - i0);
        if (!is.read(in.data(), (std::streamsize)(m * rec))) return fail("short read");
        for (uint64_t r = 0; r < m; ++r) {
            const char *p = in.data() + r * rec;
            int32_t len;
            std::memcpy(&len, p, 4);
            if (len != d)
                return fail("vector " + std::to_string(i0 + r) + " has length " + std::to_string(len) + ", expected " +
                            std::to_string(d));
            std::memcpy(out.data() + r * (uint64_t)d, p + 4, 4 * (size_t)d);
        }
        if (i0 == 0 && m > 0) {
            for (int32_t j = 0; j < d; ++j) std::cout << out[(size_t)j] << ' ';
            std::cout << std::endl;
        }
        os.write(reinterpret_cast<const char *>(out.data()), (std::streamsize)(m * 4 * (uint64_t)d));
        if (!os) return fail("write failed");
    }
    os.close();
    return os ? 0 : fail("write failed");
}
