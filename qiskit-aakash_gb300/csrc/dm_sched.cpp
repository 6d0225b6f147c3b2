// Levelling of a merged instruction list into clock cycles, with the
// reference's semantics (qiskit/providers/basicaer/basicaertools.py:714-749
// partition, built on :536-591 qubit_stack and :594-712 partition_helper).
//
// The number of levels is physics, not only scheduling: the reference
// applies memory noise to every qubit once per level
// (dm_simulator.py:1173-1177).  The algorithm, restated:
// * the list is split on barriers; each non-empty piece is levelled alone;
// * per qubit a stack of the piece's instructions in program order; a
//   measurement or reset goes on its first qubit's stack with a placeholder
//   on every qubit it does not name, and joins the placeholder on top of its
//   first qubit's stack when one of its own kind is pending there (a group of
//   simultaneous measurements / resets);
// * each level scans the qubits in order: a single-qubit gate on top of a
//   free qubit is placed; a CX is placed when it is on top of both its
//   qubits and both are free; a measurement / reset group is placed, on a
//   level of its own, once every qubit's top is empty, a placeholder of its
//   kind or an instruction of its kind;
// * a piece's level table is pre-sized to its longest stack and grows as
//   needed; the tables of the pieces are concatenated (unused trailing
//   entries included) and the first `levels` entries are executed.
// Host code only; no CUDA.
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "dm_gb300.h"

namespace {

constexpr int32_t kNone = -1000000000;

inline bool is_group(int32_t kind) { return kind == DM_SCHED_MEASURE || kind == DM_SCHED_RESET; }

// A stack entry is an instruction index (>= 0) or a placeholder -kind (kind 3 or 4).
inline bool is_placeholder(int32_t e) { return e < 0; }

struct Out {
    int32_t *inst, *pos;
    int32_t count = 0, capacity = 0;
};

int level_piece(int n, int begin, int end, const int32_t *kind, const int32_t *qoff, const int32_t *qubits,
                int32_t table_base, Out &out, int32_t *table_size_out, int32_t *levels_out) {
    std::vector<std::vector<int32_t>> stacks(static_cast<size_t>(n));
    for (int i = begin; i < end; ++i) {
        const int32_t k = kind[i];
        if (!is_group(k)) {
            for (int j = qoff[i]; j < qoff[i + 1]; ++j) stacks[size_t(qubits[j])].push_back(i);
            continue;
        }
        const int q0 = qubits[qoff[i]];
        std::vector<int32_t> &s0 = stacks[size_t(q0)];
        if (!s0.empty() && s0.back() == -k) {   // joins the pending simultaneous group
            s0.back() = i;
            continue;
        }
        s0.push_back(i);
        for (int q = 0; q < n; ++q) {
            bool named = false;
            for (int j = qoff[i]; j < qoff[i + 1]; ++j) named = named || qubits[j] == q;
            if (!named) stacks[size_t(q)].push_back(-k);
        }
    }
    size_t table_size = 0;
    for (const auto &s : stacks) table_size = s.size() > table_size ? s.size() : table_size;
    std::vector<int32_t> placed_at(table_size, 0);
    std::vector<size_t> heads(static_cast<size_t>(n), 0);
    std::vector<char> busy(static_cast<size_t>(n), 0);
    auto top = [&](int q) -> int32_t {
        const auto &s = stacks[size_t(q)];
        return heads[size_t(q)] < s.size() ? s[heads[size_t(q)]] : kNone;
    };
    auto place = [&](int32_t inst, size_t level) -> bool {
        if (out.count >= out.capacity) return false;
        out.inst[out.count] = inst;
        out.pos[out.count] = table_base + int32_t(level);
        ++out.count;
        ++placed_at[level];
        return true;
    };
    int64_t remaining = end - begin;
    size_t level = 0;
    while (remaining > 0) {
        std::fill(busy.begin(), busy.end(), 0);
        const int64_t placed_before = remaining;
        if (level == table_size) {
            ++table_size;
            placed_at.push_back(0);
        }
        for (int q = 0; q < n; ++q) {
            const int32_t g = top(q);
            if (g == kNone || is_placeholder(g)) continue;
            const int32_t k = kind[g];
            if (k == DM_SCHED_GATE1) {
                if (busy[size_t(q)]) continue;
                if (!place(g, level)) return DM_ERR_RANGE;
                busy[size_t(q)] = 1;
                ++heads[size_t(q)];
                --remaining;
            } else if (k == DM_SCHED_CX) {
                int other = -1;
                for (int j = qoff[g]; j < qoff[g + 1]; ++j)
                    if (qubits[j] != q) {
                        other = qubits[j];
                        break;
                    }
                if (other < 0 || busy[size_t(q)] || busy[size_t(other)] || top(other) != g) continue;
                if (!place(g, level)) return DM_ERR_RANGE;
                busy[size_t(q)] = busy[size_t(other)] = 1;
                ++heads[size_t(q)];
                ++heads[size_t(other)];
                --remaining;
            } else if (is_group(k)) {
                bool ready = true;
                for (int x = 0; x < n && ready; ++x) {
                    const int32_t t = top(x);
                    ready = t == kNone || (is_placeholder(t) ? t == -k : kind[t] == k);
                }
                if (!ready) continue;
                if (placed_at[level] > 0) {
                    std::fill(busy.begin(), busy.end(), 0);
                    ++level;
                    if (level == table_size) {
                        ++table_size;
                        placed_at.push_back(0);
                    }
                }
                for (int x = 0; x < n; ++x) {
                    const int32_t t = top(x);
                    if (t == kNone) continue;
                    if (!is_placeholder(t)) {
                        busy[size_t(x)] = 1;
                        if (!place(t, level)) return DM_ERR_RANGE;
                        --remaining;
                    }
                    ++heads[size_t(x)];
                }
                break;
            }
            if (remaining == 0) break;
        }
        if (remaining == placed_before) return DM_ERR_PROGRAM;   // nothing could be placed
        ++level;
    }
    *table_size_out = int32_t(table_size);
    *levels_out = int32_t(level);
    return DM_OK;
}

}  // namespace

extern "C" int dm_levelize(int n, int count, const int32_t *kind, const int32_t *qoff, const int32_t *qubits,
                           int32_t *placed_inst, int32_t *placed_pos, int32_t *placed_count, int32_t *table_len,
                           int32_t *levels) {
    if (n < 1 || count < 0 || (count > 0 && (!kind || !qoff || !qubits)) || !placed_count || !table_len || !levels)
        return DM_ERR_ARG;
    if (count > 0 && (!placed_inst || !placed_pos)) return DM_ERR_ARG;
    if (count > 0 && qoff[0] != 0) return DM_ERR_ARG;
    for (int i = 0; i < count; ++i) {
        if (qoff[i + 1] < qoff[i]) return DM_ERR_ARG;
        if (kind[i] < DM_SCHED_GATE1 || kind[i] > DM_SCHED_OTHER) return DM_ERR_ARG;
        if (kind[i] != DM_SCHED_BARRIER && qoff[i + 1] == qoff[i]) return DM_ERR_ARG;
        for (int j = qoff[i]; j < qoff[i + 1]; ++j)
            if (qubits[j] < 0 || qubits[j] >= n) return DM_ERR_ARG;
        if (kind[i] == DM_SCHED_GATE1 && qoff[i + 1] - qoff[i] != 1) return DM_ERR_ARG;
    }
    Out out;
    out.inst = placed_inst;
    out.pos = placed_pos;
    out.capacity = count;
    int32_t table = 0, lv = 0;
    int begin = 0;
    for (int i = 0; i <= count; ++i) {
        if (i < count && kind[i] != DM_SCHED_BARRIER) continue;
        if (i > begin) {
            int32_t ts = 0, pl = 0;
            const int rc = level_piece(n, begin, i, kind, qoff, qubits, table, out, &ts, &pl);
            if (rc) return rc;
            table += ts;
            lv += pl;
        }
        begin = i + 1;
    }
    *placed_count = out.count;
    *table_len = table;
    *levels = lv;
    return DM_OK;
}
