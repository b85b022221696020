// Host build of textscan.cuh for tests/test_textscan_cpu.py: reads one field per line from stdin as
// "<kind> <hex bytes>" (kind: i = integer, f = double, d = DATE32, t = DATE64) and prints
// "<status> <value>" (the value's 64-bit pattern for doubles, the integer otherwise).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "textscan.cuh"

static int hexval(char c) { return c <= '9' ? c - '0' : (c | 0x20) - 'a' + 10; }

int main() {
    char line[1 << 16];
    std::vector<char> buf;
    while (std::fgets(line, sizeof line, stdin)) {
        const char kind = line[0];
        buf.clear();
        for (const char* p = line + 2; p[0] && p[0] != '\n' && p[1]; p += 2)
            buf.push_back((char)(hexval(p[0]) * 16 + hexval(p[1])));
        const char* s = buf.data();
        const long long n = (long long)buf.size();
        int st = 0;
        long long iv = 0;
        double dv = 0;
        switch (kind) {
        case 'i': st = ral_tx_parse_int(s, 0, n, &iv); break;
        case 'f': st = ral_tx_parse_double(s, 0, n, &dv); std::memcpy(&iv, &dv, 8); break;
        case 'd': st = ral_tx_parse_date(s, 0, n, false, &iv); break;
        default: st = ral_tx_parse_date(s, 0, n, true, &iv); break;
        }
        std::printf("%d %lld\n", st, st == RAL_TX_OK ? iv : 0ll);
    }
    return 0;
}
