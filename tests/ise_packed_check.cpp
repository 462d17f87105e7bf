// Host harness for the rolled ISE encoder (astc_ise.h): reads lines
// "quant count v0 .. v{count-1}" from stdin and prints the 16 encoded bytes
// of each as hex.  Built and driven by test_ise_packed.py.
#include <cstdio>
#include <cstdint>
#include "astc_ise.h"

int main() {
    const astc::IseTables t = astc::make_ise_tables();
    int quant, count;
    while (std::scanf("%d %d", &quant, &count) == 2) {
        uint32_t v[32] = {0};
        for (int i = 0; i < count && i < 32; ++i)
            if (std::scanf("%u", &v[i]) != 1) return 1;
        uint32_t w[8];
        astc::pack_bytes<32>(v, w);
        const astc::Bits128 o = astc::ise_encode_packed<8>(quant, count, w, t.trit_pack, t.quint_pack);
        for (int i = 0; i < 16; ++i)
            std::printf("%02x", (unsigned)((i < 8 ? o.lo >> (8 * i) : o.hi >> (8 * (i - 8))) & 0xFFu));
        std::printf("\n");
    }
    return 0;
}
