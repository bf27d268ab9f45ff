// No-op replacement for the reference's console progress reporter
// (libSLR/Core/ProgressReporter.cpp).  TEST INFRASTRUCTURE ONLY: it is linked
// into the CPU oracle instead of the stock reporter, whose print thread makes
// popJob() wait up to 250 ms per progressive pass (ProgressReporter.cpp:74-81)
// and whose unsynchronised work counter (ProgressReporter.cpp:101-104) can
// leave render() waiting forever.  The interface is the one declared in
// libSLR/Core/ProgressReporter.h; elapsed() keeps working because the job
// stack still records each job's start time.
#include "Core/ProgressReporter.h"

namespace SLR {
    ProgressReporter::ProgressReporter() : m_sleep(true), m_numLastLines(0), m_finishable(false) {}

    void ProgressReporter::pushJob(const std::string &title, uint64_t totalWork,
                                   const std::chrono::system_clock::time_point &startTime) {
        std::lock_guard<std::mutex> lock(m_jobMutex);
        m_jobStask.emplace_back(title, totalWork, startTime);
    }

    void ProgressReporter::popJob() {
        std::lock_guard<std::mutex> lock(m_jobMutex);
        if (m_jobStask.size() > 1)
            m_jobStask.pop_back();
    }

    void ProgressReporter::beginOtherThreadPrint() {}
    void ProgressReporter::endOtherThreadPrint() {}
    void ProgressReporter::update(uint64_t) {}
    void ProgressReporter::finish() {}
}
