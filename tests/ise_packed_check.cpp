// Host harness for the ISE encoders of astc_ise.h: reads lines
// "form quant count v0 .. v{count-1}" from stdin (form 0: the rolled loop,
// 1: the compile-time form of the range, for counts 6, 8, 12, 16, 18 and 32)
// and prints the 16 encoded bytes of each as hex.  Built and driven by
// test_ise_packed.py.
#include <cstdint>
#include <cstdio>

#include "astc_ise.h"

namespace {

const astc::IseTables& tables() {
    static const astc::IseTables t = astc::make_ise_tables();
    return t;
}

template <int COUNT>
astc::Bits128 fixed_form(int quant, const uint32_t* in) {
    uint32_t v[COUNT];
    for (int i = 0; i < COUNT; ++i) v[i] = in[i];
    return astc::ise_encode_chain<COUNT, astc::kQuant2, astc::kQuant256>(quant, v, tables().trit_pack,
                                                                          tables().quint_pack);
}

}  // namespace

int main() {
    int form, quant, count;
    while (std::scanf("%d %d %d", &form, &quant, &count) == 3) {
        uint32_t v[32] = {0};
        for (int i = 0; i < count && i < 32; ++i)
            if (std::scanf("%u", &v[i]) != 1) return 1;
        astc::Bits128 o{0, 0};
        if (form == 0) {
            uint32_t w[8];
            astc::pack_bytes<32>(v, w);
            o = astc::ise_encode_packed<8>(quant, count, w, tables().trit_pack, tables().quint_pack);
        } else {
            switch (count) {
                case 6: o = fixed_form<6>(quant, v); break;
                case 8: o = fixed_form<8>(quant, v); break;
                case 12: o = fixed_form<12>(quant, v); break;
                case 16: o = fixed_form<16>(quant, v); break;
                case 18: o = fixed_form<18>(quant, v); break;
                case 32: o = fixed_form<32>(quant, v); break;
                default: return 2;
            }
        }
        for (int i = 0; i < 16; ++i)
            std::printf("%02x", (unsigned)((i < 8 ? o.lo >> (8 * i) : o.hi >> (8 * (i - 8))) & 0xFFu));
        std::printf("\n");
    }
    return 0;
}
