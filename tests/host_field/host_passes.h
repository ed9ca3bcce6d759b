// The device pass sequence of a frame, run on the host item by item (tests/host_checks.py):
// for each reflection level, the march (march_kernels.cuh m_start / m_step), the next level's
// reflection rays, AO, soft shadows and shading (shade_kernels.cuh), as the engine launches them.
// Every level keeps its own queue and hit records, as the device keeps the primary level's apart
// from the reflection levels' (its resolve and G-buffer read the primary records). Include after
// shade_kernels.cuh. Test infrastructure only.
#pragma once
#include <vector>

struct HostFrame {
    uint32_t cap = 0, levels = 0, nl = 0;
    std::vector<std::vector<float4>> q_o, q_d, h_n;
    std::vector<std::vector<uint2>> h_m;
    std::vector<std::vector<float>> occ, shadow;
    std::vector<float4> term, lvl, hdr, fg;
    uint32_t nq_count = 0;

    void init(uint32_t cap_, uint32_t levels_, uint32_t nl_, uint32_t pixels) {
        cap = cap_;
        levels = levels_;
        nl = nl_;
        q_o.assign(levels, std::vector<float4>(cap));
        q_d.assign(levels, std::vector<float4>(cap));
        h_n.assign(levels, std::vector<float4>(cap));
        h_m.assign(levels, std::vector<uint2>(cap));
        occ.assign(levels, std::vector<float>(cap));
        shadow.assign(levels, std::vector<float>((size_t)cap * (nl ? nl : 1u)));
        term.assign(cap, make_float4(0.f, 0.f, 0.f, 0.f));
        lvl.assign((size_t)2 * cap * levels, make_float4(0.f, 0.f, 0.f, 0.f));
        hdr.assign(pixels, make_float4(0.f, 0.f, 0.f, 0.f));
        fg.assign(pixels, make_float4(0.f, 0.f, 0.f, 0.f));
    }

    // Point the pass arguments at level `level`'s queue and records.
    void bind(mm3e::WaveArgs& a, uint32_t level) {
        a.b.q_o = q_o[level].data();
        a.b.q_d = q_d[level].data();
        a.b.h_n = h_n[level].data();
        a.b.h_m = h_m[level].data();
        a.b.occ = occ[level].data();
        a.b.shadow = shadow[level].data();
        a.b.nq_o = level + 1 < levels ? q_o[level + 1].data() : nullptr;
        a.b.nq_d = level + 1 < levels ? q_d[level + 1].data() : nullptr;
        a.b.nq_count = &nq_count;
        a.b.term = term.data();
        a.b.lvl = lvl.data();
        a.b.hdr = hdr.data();
        a.b.fg = fg.data();
        a.cap = cap;
        a.lights_max = nl;
    }
};

// Every level of one pass sequence: level 0 takes `n0` items from `src0` (the jobs' camera
// samples, or a queue already in F.q_o[0] / F.q_d[0]); the AO and shadow passes run when `ao` /
// `shadows` say so (for a job table: when any job needs them). `tape` is the lanes' first tape
// (each item then takes its own job's). Leaves `a` bound to level 0.
template <class FP>
void host_levels_with(mm3e::WaveArgs& a, const unsigned char* tape, uint32_t src0, uint32_t n0, HostFrame& F, bool ao,
                      bool shadows) {
    using namespace mm3e;
    using namespace mm3e::wave;
    uint32_t n = n0;
    for (uint32_t level = 0; level < F.levels && n > 0; ++level) {
        F.bind(a, level);
        a.level = level;
        a.src = level == 0 ? src0 : SRC_QUEUE;
        a.n_items = n;
        for (uint32_t i = 0; i < n; ++i) {
            MLane L;
            L.item = i;
            L.phase = M_IDLE;
            LaneTape<TM_MULTI> LT;
            LT.p = tape;
            if (m_start<TM_MULTI, FP>(L, LT, a))
                while (L.phase != M_IDLE) m_step<TM_MULTI, FP>(L, LT, a);
        }
        F.nq_count = 0;
        if (level + 1 < F.levels)
            for (uint32_t i = 0; i < n; ++i) reflect_slots(a, i, true);
        if (ao)
            for (uint32_t i = 0; i < n; ++i) ao_slot<FP>(a, i);
        if (shadows)
            for (uint32_t i = 0; i < n * F.nl; ++i) {
                SLane S;
                S.item = i;
                LaneTape<TM_MULTI> LT;
                LT.p = tape;
                if (s_start<TM_MULTI, FP>(S, LT, a, n))
                    while (S.item != NIL) s_step<TM_MULTI, FP>(S, LT, a);
            }
        for (uint32_t i = 0; i < n; ++i) shade_slots(a, i, true);
        n = F.nq_count;
    }
    F.bind(a, 0);
}

// One scene's pass sequence: its AO and shadow passes run as the engine's plan decides.
template <class FP>
void host_levels(mm3e::WaveArgs& a, const unsigned char* tape, uint32_t src0, uint32_t n0, HostFrame& F) {
    using namespace mm3e;
    const TapeHeader& H = *tape_view(tape).h;
    host_levels_with<FP>(a, tape, src0, n0, F, (H.flags & SF_AO) && H.ao_samples > 0,
                         (H.flags & SF_SHADOWS) && H.shadow_steps > 0 && F.nl > 0);
}
