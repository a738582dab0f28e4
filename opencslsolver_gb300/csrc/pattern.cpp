// Host-side analysis of the fixed CSR pattern (done once per run, like the
// reference's CFVM::define_matrix_structure, cfvm.cpp:74-98).
//
// Produces everything the device needs besides values:
//   * int32 CSR with the phantom column (size_t)-1 mapped to -1;
//   * the diagonal positions (extract_diag_indexes, cmatrix_solver.cpp:455-469);
//   * the ILU product table: for stored entry j of row i, the pairs (k, slot)
//     such that the reference's sweep (cmatrix_solver.cpp:527-547) adds
//     M[k] * M.get_element(col[k], col[j]) with a match at `slot`, in the
//     reference's k order; products whose get_element finds nothing add an
//     exact 0 and are left out;
//   * level schedules of the forward (strict lower part) and backward
//     (strict upper part) sweeps, each level cut into chunks of <= 256 rows.
#include "pattern.h"

#include <algorithm>
#include <climits>
#include <cstdio>

namespace ocsl {

namespace {

constexpr uint64_t kPhantom = ~uint64_t(0);

bool fail(std::string& err, const char* fmt, long long a, long long b = 0)
{
    char buf[256];
    std::snprintf(buf, sizeof buf, fmt, a, b);
    err = buf;
    return false;
}

void schedule(int n, const std::vector<int>& level, int nlevels, std::vector<int>& order,
              std::vector<int>& chunk, std::vector<int>& range, int chunk_rows)
{
    std::vector<int> count(nlevels + 1, 0);
    for (int i = 0; i < n; ++i) ++count[level[i] + 1];
    for (int l = 0; l < nlevels; ++l) count[l + 1] += count[l];
    std::vector<int> start(count.begin(), count.end() - 1);
    order.assign(n, 0);
    for (int i = 0; i < n; ++i) order[start[level[i]]++] = i;  // ascending rows per level
    chunk.clear();
    for (int l = 0; l < nlevels; ++l) {
        for (int b = count[l]; b < count[l + 1]; b += chunk_rows) chunk.push_back(b);
    }
    chunk.push_back(n);
    // levels that are contiguous row ranges (rows ascend within a level, so
    // the first and last row tell)
    range.clear();
    if (nlevels > kRangeMaxLevels) return;
    for (int l = 0; l < nlevels; ++l) {
        const int a = count[l], b = count[l + 1];
        if (b > a && order[b - 1] - order[a] != b - 1 - a) {
            range.clear();
            return;
        }
        range.push_back(b > a ? order[a] : 0);
        range.push_back(b > a ? order[b - 1] + 1 : 0);
    }
}

}  // namespace

BoxShape detect_box(int n, const std::vector<int>& rp, const std::vector<int>& col)
{
    BoxShape none;
    if (n < 2) return none;
    // Row 0's real upper columns give the strides: [1], [1, nx] or [1, nx, nx*ny].
    std::vector<long long> up;
    for (int q = rp[0]; q < rp[1]; ++q)
        if (col[q] > 0) up.push_back(col[q]);
    long long nx, ny, nz;
    if (up.size() == 1 && up[0] == 1) {
        nx = n; ny = 1; nz = 1;
    } else if (up.size() == 2 && up[0] == 1 && up[1] > 1 && n % up[1] == 0) {
        nx = up[1]; ny = n / up[1]; nz = 1;
    } else if (up.size() == 3 && up[0] == 1 && up[1] > 1 && up[2] % up[1] == 0 && up[2] > up[1] &&
               n % up[2] == 0) {
        nx = up[1]; ny = up[2] / up[1]; nz = n / up[2];
    } else {
        return none;
    }
    const long long nxy = nx * ny;
    for (int r = 0; r < n; ++r) {
        const long long i = r % nx, j = (r / nx) % ny, k = r / nxy;
        long long want[7];
        int m = 0;
        if (k > 0) want[m++] = r - nxy;
        if (j > 0) want[m++] = r - nx;
        if (i > 0) want[m++] = r - 1;
        want[m++] = r;
        if (i < nx - 1) want[m++] = r + 1;
        if (j < ny - 1) want[m++] = r + nx;
        if (k < nz - 1) want[m++] = r + nxy;
        int q = rp[r], t = 0;
        for (; q < rp[r + 1] && col[q] >= 0; ++q, ++t)
            if (t >= m || col[q] != want[t]) return none;
        if (t != m) return none;
        for (; q < rp[r + 1]; ++q)
            if (col[q] >= 0) return none;  // only phantoms may follow
    }
    BoxShape b;
    b.ok = true;
    b.dim[0] = (int)nx;
    b.dim[1] = (int)ny;
    b.dim[2] = (int)nz;
    return b;
}

bool analyse_pattern(size_t n_in, const size_t* rp, const size_t* col, HostPattern& hp,
                     std::string& err)
{
    if (n_in >= (size_t)INT_MAX) return fail(err, "n = %lld exceeds the int32 limit", (long long)n_in);
    const int n = (int)n_in;
    hp = HostPattern();
    hp.n = n;
    if (n == 0) {
        hp.rp.assign(1, 0);
        hp.fw_chunk.assign(1, 0);
        hp.bw_chunk.assign(1, 0);
        hp.pair_ptr.assign(1, 0);
        return true;
    }
    if (!rp || !col) return fail(err, "null row_ptr or column_index (n = %lld)", n);
    if (rp[0] != 0) return fail(err, "row_ptr[0] = %lld, expected 0", (long long)rp[0]);
    for (int i = 0; i < n; ++i)
        if (rp[i + 1] < rp[i]) return fail(err, "row_ptr decreases at row %lld", i);
    if (rp[n] >= (size_t)INT_MAX) return fail(err, "nnz = %lld exceeds the int32 limit", (long long)rp[n]);
    const int nnz = (int)rp[n];
    hp.nnz = nnz;
    hp.rp.resize(n + 1);
    hp.col.resize(nnz);
    hp.diag.resize(n);
    for (int i = 0; i <= n; ++i) hp.rp[i] = (int)rp[i];

    for (int i = 0; i < n; ++i) {
        int d = -1;
        for (int q = hp.rp[i]; q < hp.rp[i + 1]; ++q) {
            const uint64_t c = col[q];
            if (c >= (uint64_t)n && c != kPhantom)
                return fail(err, "row %lld: column %lld out of range", i, (long long)c);
            hp.col[q] = c == kPhantom ? -1 : (int)c;
            if (c != kPhantom) ++hp.nnz_real;
            if (d < 0 && c == (uint64_t)i) d = q;
        }
        if (d < 0) return fail(err, "row %lld has no diagonal entry", i);
        hp.diag[i] = d;
        for (int q = hp.rp[i]; q < d; ++q)
            if (!(col[q] < (uint64_t)i))
                return fail(err, "row %lld: entry before the diagonal is not below it (col %lld)", i,
                            (long long)col[q]);
        for (int q = d + 1; q < hp.rp[i + 1]; ++q)
            if (!(col[q] > (uint64_t)i))
                return fail(err, "row %lld: entry after the diagonal is not above it (col %lld)", i,
                            (long long)col[q]);
    }

    // ILU product table.
    hp.pair_ptr.assign(nnz + 1, 0);
    hp.pair_k.clear();
    hp.pair_slot.clear();
    for (int i = 0; i < n; ++i) {
        const int b = hp.rp[i], e = hp.rp[i + 1], d = hp.diag[i];
        for (int j = b; j < e; ++j) {
            const uint64_t cj = col[j];
            const bool lower = cj != kPhantom && (uint64_t)i > cj;
            const int kend = lower ? j : d;
            for (int k = b; k < kend; ++k) {
                const uint64_t r = col[k];  // a row index: entries before the diagonal are < i
                int slot = -1;
                for (size_t q = rp[r]; q < rp[r + 1]; ++q)
                    if (col[q] == cj) { slot = (int)q; break; }
                if (slot >= 0) {
                    if (hp.pair_k.size() >= (size_t)INT_MAX)
                        return fail(err, "ILU product table exceeds the int32 limit at row %lld", i);
                    hp.pair_k.push_back(k);
                    hp.pair_slot.push_back(slot);
                }
            }
            hp.pair_ptr[j + 1] = (int)hp.pair_k.size();
        }
    }

    // Level schedules.
    std::vector<int> level(n, 0);
    int nl = 0;
    for (int i = 0; i < n; ++i) {
        int l = 0;
        for (int q = hp.rp[i]; q < hp.diag[i]; ++q) l = std::max(l, level[hp.col[q]] + 1);
        level[i] = l;
        nl = std::max(nl, l + 1);
    }
    hp.fw_levels = nl;
    schedule(n, level, nl, hp.fw_order, hp.fw_chunk, hp.fw_range, kChunkRows);
    nl = 0;
    for (int i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int q = hp.diag[i] + 1; q < hp.rp[i + 1]; ++q)
            if (hp.col[q] >= 0) l = std::max(l, level[hp.col[q]] + 1);
        level[i] = l;
        nl = std::max(nl, l + 1);
    }
    hp.bw_levels = nl;
    schedule(n, level, nl, hp.bw_order, hp.bw_chunk, hp.bw_range, kChunkRows);
    hp.box = detect_box(n, hp.rp, hp.col);
    return true;
}

bool build_face_tables(int n, const std::vector<int>& rp, const std::vector<int>& col,
                       long long nf, const int32_t* left, const int32_t* right, long long nb,
                       const int32_t* bc_left, FaceTables& ft, std::string& err)
{
    if (nf < 0 || nb < 0 || nf >= (1LL << 30) || nb >= INT_MAX)
        return fail(err, "face counts out of range (%lld, %lld)", nf, nb);
    auto find = [&](int i, int j) {
        for (int q = rp[i]; q < rp[i + 1]; ++q)
            if (col[q] == j) return q;
        return -1;
    };
    ft = FaceTables();
    std::vector<int> cnt(n + 1, 0), bcnt(n + 1, 0);
    for (long long f = 0; f < nf; ++f) {
        const int L = left[f], R = right[f];
        if (L < 0 || L >= n || R < 0 || R >= n || L == R)
            return fail(err, "interior face %lld joins cells out of range or itself (%lld)", f, L);
        ++cnt[L + 1];
        ++cnt[R + 1];
    }
    for (long long g = 0; g < nb; ++g) {
        if (bc_left[g] < 0 || bc_left[g] >= n)
            return fail(err, "boundary face %lld names cell %lld", g, bc_left[g]);
        ++bcnt[bc_left[g] + 1];
    }
    for (int i = 0; i < n; ++i) {
        cnt[i + 1] += cnt[i];
        bcnt[i + 1] += bcnt[i];
    }
    ft.cell_ptr = cnt;
    ft.bc_ptr = bcnt;
    ft.cell_ent.assign(cnt[n], 0);
    ft.cell_slot.assign(cnt[n], 0);
    ft.bc_ent.assign(bcnt[n], 0);
    std::vector<int> next(cnt.begin(), cnt.end() - 1), bnext(bcnt.begin(), bcnt.end() - 1);
    for (long long f = 0; f < nf; ++f) {  // ascending f keeps every list in face order
        const int L = left[f], R = right[f];
        const int kLR = find(L, R), kRL = find(R, L);
        if (kLR < 0 || kRL < 0)
            return fail(err, "face %lld: pair (%lld, right) is not in the pattern", f, L);
        int e = next[L]++;
        ft.cell_ent[e] = (int)(f << 1);
        ft.cell_slot[e] = kLR;
        e = next[R]++;
        ft.cell_ent[e] = (int)(f << 1) | 1;
        ft.cell_slot[e] = kRL;
    }
    for (long long g = 0; g < nb; ++g) ft.bc_ent[bnext[bc_left[g]]++] = (int)g;
    return true;
}

bool build_pattern_from_faces(size_t n, long long nf, const int32_t* left, const int32_t* right,
                              long long nb, const int32_t* bc_left, std::vector<size_t>& row_ptr,
                              std::vector<size_t>& column_index, std::string& err)
{
    if (n >= (size_t)INT_MAX) return fail(err, "n = %lld exceeds the int32 limit", (long long)n);
    const long long N = (long long)n;
    std::vector<int> deg(n + 1, 0);
    std::vector<char> boundary(n, 0);
    for (long long f = 0; f < nf; ++f) {
        if (left[f] < 0 || left[f] >= N || right[f] < 0 || right[f] >= N)
            return fail(err, "interior face %lld names a cell out of range", f);
        ++deg[left[f] + 1];
        ++deg[right[f] + 1];
    }
    for (long long g = 0; g < nb; ++g) {
        if (bc_left[g] < 0 || bc_left[g] >= N)
            return fail(err, "boundary face %lld names a cell out of range", g);
        boundary[bc_left[g]] = 1;
    }
    for (size_t i = 0; i < n; ++i) deg[i + 1] += deg[i];
    std::vector<int> nbr(deg[n]);
    std::vector<int> next(deg.begin(), deg.end() - 1);
    for (long long f = 0; f < nf; ++f) {
        nbr[next[left[f]]++] = right[f];
        nbr[next[right[f]]++] = left[f];
    }
    row_ptr.assign(n + 1, 0);
    column_index.clear();
    column_index.reserve((size_t)deg[n] + 2 * n);
    std::vector<int> cols;
    for (size_t i = 0; i < n; ++i) {
        cols.assign(nbr.begin() + deg[i], nbr.begin() + deg[i + 1]);
        cols.push_back((int)i);
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());  // repeated pairs merge
        for (int c : cols) column_index.push_back((size_t)c);
        if (boundary[i]) column_index.push_back(~size_t(0));  // one phantom per boundary cell
        row_ptr[i + 1] = column_index.size();
    }
    return true;
}

bool colour_pattern(int n, const std::vector<int>& rp, const std::vector<int>& col,
                    ColouredPattern& cp, std::string& err)
{
    cp = ColouredPattern();
    std::vector<int> colour(n, -1);
    std::vector<int> seen;  // seen[c] == i: colour c is taken by a neighbour of row i
    int nc = 0;
    for (int i = 0; i < n; ++i) {
        for (int q = rp[i]; q < rp[i + 1]; ++q) {
            const int j = col[q];
            if (j >= 0 && j != i && colour[j] >= 0) {
                if ((int)seen.size() <= colour[j]) seen.resize(colour[j] + 1, -1);
                seen[colour[j]] = i;
            }
        }
        int c = 0;
        while (c < (int)seen.size() && seen[c] == i) ++c;
        colour[i] = c;
        nc = std::max(nc, c + 1);
    }
    // a neighbour with the same colour means the pattern is not symmetric
    for (int i = 0; i < n; ++i)
        for (int q = rp[i]; q < rp[i + 1]; ++q)
            if (col[q] >= 0 && col[q] != i && colour[col[q]] == colour[i])
                return fail(err, "rows %lld and %lld: the pattern is not structurally symmetric",
                            i, col[q]);
    cp.colours = nc;
    std::vector<int> start(nc + 1, 0), inv(n);
    for (int i = 0; i < n; ++i) ++start[colour[i] + 1];
    for (int c = 0; c < nc; ++c) start[c + 1] += start[c];
    cp.start = start;
    cp.perm.resize(n);
    for (int i = 0; i < n; ++i) {
        const int k = start[colour[i]]++;
        cp.perm[k] = i;
        inv[i] = k;
    }
    cp.rp.assign(n + 1, 0);
    cp.col.reserve(col.size());
    cp.slot.reserve(col.size());
    std::vector<std::pair<int, int>> row;  // (new column, old slot)
    std::vector<int> phantoms;
    for (int k = 0; k < n; ++k) {
        const int i = cp.perm[k];
        row.clear();
        phantoms.clear();
        for (int q = rp[i]; q < rp[i + 1]; ++q) {
            if (col[q] < 0)
                phantoms.push_back(q);
            else
                row.push_back({inv[col[q]], q});
        }
        std::sort(row.begin(), row.end());
        for (const auto& e : row) {
            cp.col.push_back((size_t)e.first);
            cp.slot.push_back(e.second);
        }
        for (int q : phantoms) {  // phantom columns stay after the real ones
            cp.col.push_back(kPhantom);
            cp.slot.push_back(q);
        }
        cp.rp[k + 1] = cp.col.size();
    }
    return true;
}

}  // namespace ocsl
