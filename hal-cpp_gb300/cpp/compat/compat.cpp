// Out-of-line members of the stand-in interface and Logger declarations
// (only linked when the backend is built outside a HAL-CPP tree).
#include "Hal/Agents/IAgentForceBackend2D.h"
#include "Hal/Log/Logger.h"
#include "Hal/Pde/IAdiDiffusionBackend2D.h"
#include "Hal/Pde/IDiffusionBackend2D.h"

#include <cstdio>

namespace Hal
{
    IDiffusionBackend2D::IDiffusionBackend2D() = default;
    IDiffusionBackend2D::~IDiffusionBackend2D() = default;
    IAdiDiffusionBackend2D::IAdiDiffusionBackend2D() = default;
    IAdiDiffusionBackend2D::~IAdiDiffusionBackend2D() = default;
    IAgentForceBackend2D::IAgentForceBackend2D() = default;
    IAgentForceBackend2D::~IAgentForceBackend2D() = default;

    Logger &Logger::Instance()
    {
        static Logger logger;
        return logger;
    }

    void Logger::Log(LogSeverity severity, const std::string &message)
    {
        if (severity < m_minSeverity)
        {
            return;
        }
        std::fprintf(stderr, "[%s] %s\n", severity == LogSeverity::Error ? "Error" : "Warning", message.c_str());
    }

    void Logger::SetMinSeverity(LogSeverity severity)
    {
        m_minSeverity = severity;
    }
}
