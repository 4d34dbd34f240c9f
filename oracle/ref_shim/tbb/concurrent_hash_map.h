// TBB-compatible shim (test infrastructure): concurrent_hash_map with locking accessors.
#ifndef FG_TBB_SHIM_CHM_H
#define FG_TBB_SHIM_CHM_H
#include <memory>
#include <mutex>
#include <unordered_map>
#include <utility>
namespace tbb {
template<typename K, typename V> class concurrent_hash_map
{
public:
    using value_type = std::pair<const K, V>;
    class const_accessor
    {
    public:
        const_accessor() = default;
        const value_type* operator->() const { return m_item; }
        const value_type& operator*() const { return *m_item; }
        void release()
        {
            m_item = nullptr;
            if (m_lock.owns_lock())
            {
                m_lock.unlock();
            }
        }
    protected:
        friend class concurrent_hash_map;
        value_type* m_item {nullptr};
        std::unique_lock<std::recursive_mutex> m_lock;
    };
    class accessor : public const_accessor
    {
    public:
        value_type* operator->() const { return this->m_item; }
        value_type& operator*() const { return *this->m_item; }
    };

    concurrent_hash_map() : m_mutex(std::make_unique<std::recursive_mutex>()) {}

    bool find(const_accessor& a, const K& key) const
    {
        a.release();
        std::unique_lock<std::recursive_mutex> lock(*m_mutex);
        auto it = m_map.find(key);
        if (it == m_map.end())
        {
            return false;
        }
        a.m_item = const_cast<value_type*>(&*it);
        a.m_lock = std::move(lock);
        return true;
    }
    bool insert(accessor& a, const K& key)
    {
        a.release();
        std::unique_lock<std::recursive_mutex> lock(*m_mutex);
        auto res = m_map.emplace(key, V());
        a.m_item = &*res.first;
        a.m_lock = std::move(lock);
        return res.second;
    }
    std::size_t size() const { return m_map.size(); }

private:
    std::unordered_map<K, V> m_map;
    std::unique_ptr<std::recursive_mutex> m_mutex;
};
}; // namespace tbb
#endif
