// Oracle build only: stand-in for oneTBB's task_arena (system TBB is not in this
// image).  The reference wraps its parallel std::sort calls in execute(); with one
// worker thread the reference never enters those calls, so a direct call suffices.
#pragma once
namespace tbb {
class task_arena {
public:
    explicit task_arena(int = 0) {}
    template <typename F>
    void execute(F&& f) { f(); }
};
}  // namespace tbb
