#pragma once

// Stand-in for HAL-CPP's include/Hal/Log/Logger.h (:8-27), used only outside
// a HAL-CPP tree: the same Instance()/Log() surface, printing errors and
// warnings to stderr.
#include <cstdint>
#include <string>

namespace Hal
{
    enum class LogSeverity : uint32_t
    {
        Debug,
        Info,
        Warning,
        Error
    };

    class Logger
    {
    public:
        static Logger &Instance();
        void Log(LogSeverity severity, const std::string &message);
        void SetMinSeverity(LogSeverity severity);

    private:
        LogSeverity m_minSeverity = LogSeverity::Warning;
    };
}
