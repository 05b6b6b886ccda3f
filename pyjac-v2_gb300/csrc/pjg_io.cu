// Binary initial-condition files, the format the reference's generated
// programs read (pyjac/kernel_utils/common/read_initial_conditions.cpp.in:30-116):
// one record of NN + 1 doubles per state, C order on disk,
//   [T, param, phi_1 (the extra variable: V for conp, P for conv), n_0 .. n_{Ns-2}],
// where param is P for constant pressure and V for constant volume.  Host code
// only; errors are returned, not fatal (the reference prints and exits).
#include <cstdint>
#include <cstdio>
#include <vector>

#include "../../include/pyjac_gb300.h"

int pjg_internal_fail(int code, const char* msg);

namespace {

constexpr int64_t kRecordsPerBlock = 4096;  // records moved per fread / fwrite

int check_args(const char* filename, int64_t n, int32_t nn, char order, const void* param,
               const void* phi)
{
    if (!filename) return pjg_internal_fail(PJG_ERR_ARG, "null file name");
    if (n < 0 || nn < 2) return pjg_internal_fail(PJG_ERR_ARG, "bad problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n > 0 && (!param || !phi)) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    return 0;
}

}  // namespace

extern "C" int pjg_read_initial_conditions(const char* filename, int64_t n, int32_t nn, char order,
                                           double* param, double* phi)
{
    int rc = check_args(filename, n, nn, order, param, phi);
    if (rc) return rc;
    FILE* fp = fopen(filename, "rb");
    if (!fp) {
        char msg[512];
        snprintf(msg, sizeof(msg), "could not open initial-conditions file %s", filename);
        return pjg_internal_fail(PJG_ERR_ARG, msg);
    }
    const int64_t rec = nn + 1;
    std::vector<double> buf((size_t)(kRecordsPerBlock * rec));
    for (int64_t s0 = 0; s0 < n; s0 += kRecordsPerBlock) {
        const int64_t cnt = n - s0 < kRecordsPerBlock ? n - s0 : kRecordsPerBlock;
        const size_t got = fread(buf.data(), sizeof(double), (size_t)(cnt * rec), fp);
        if (got != (size_t)(cnt * rec)) {
            fclose(fp);
            char msg[512];
            snprintf(msg, sizeof(msg),
                     "initial-conditions file %s is incorrectly formatted: %lld doubles were "
                     "expected but only %lld were read",
                     filename, (long long)(n * rec), (long long)(s0 * rec + (int64_t)got));
            return pjg_internal_fail(PJG_ERR_ARG, msg);
        }
        for (int64_t l = 0; l < cnt; ++l) {
            const double* r = buf.data() + l * rec;
            const int64_t s = s0 + l;
            param[s] = r[1];
            if (order == 'C') {
                phi[s * nn] = r[0];
                for (int32_t j = 1; j < nn; ++j) phi[s * nn + j] = r[j + 1];
            } else {
                phi[s] = r[0];
                for (int32_t j = 1; j < nn; ++j) phi[s + n * j] = r[j + 1];
            }
        }
    }
    fclose(fp);
    return 0;
}

extern "C" int pjg_write_initial_conditions(const char* filename, int64_t n, int32_t nn, char order,
                                            const double* param, const double* phi)
{
    int rc = check_args(filename, n, nn, order, param, phi);
    if (rc) return rc;
    FILE* fp = fopen(filename, "wb");
    if (!fp) {
        char msg[512];
        snprintf(msg, sizeof(msg), "could not create initial-conditions file %s", filename);
        return pjg_internal_fail(PJG_ERR_ARG, msg);
    }
    const int64_t rec = nn + 1;
    std::vector<double> buf((size_t)(kRecordsPerBlock * rec));
    for (int64_t s0 = 0; s0 < n; s0 += kRecordsPerBlock) {
        const int64_t cnt = n - s0 < kRecordsPerBlock ? n - s0 : kRecordsPerBlock;
        for (int64_t l = 0; l < cnt; ++l) {
            double* r = buf.data() + l * rec;
            const int64_t s = s0 + l;
            r[1] = param[s];
            if (order == 'C') {
                r[0] = phi[s * nn];
                for (int32_t j = 1; j < nn; ++j) r[j + 1] = phi[s * nn + j];
            } else {
                r[0] = phi[s];
                for (int32_t j = 1; j < nn; ++j) r[j + 1] = phi[s + n * j];
            }
        }
        if (fwrite(buf.data(), sizeof(double), (size_t)(cnt * rec), fp) != (size_t)(cnt * rec)) {
            fclose(fp);
            return pjg_internal_fail(PJG_ERR_ARG, "write to the initial-conditions file failed");
        }
    }
    if (fclose(fp) != 0) return pjg_internal_fail(PJG_ERR_ARG, "closing the initial-conditions file failed");
    return 0;
}
