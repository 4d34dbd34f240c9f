// TBB-compatible shim (test infrastructure): enumerable_thread_specific and flatten2d.
#ifndef FG_TBB_SHIM_ETS_H
#define FG_TBB_SHIM_ETS_H
#include <atomic>
#include <cstdint>
#include <deque>
#include <functional>
#include <iterator>
#include <map>
#include <mutex>
#include <thread>
#include <type_traits>
#include <utility>
namespace tbb {
template<typename T> class enumerable_thread_specific
{
public:
    using container = std::deque<T>;
    using iterator = typename container::iterator;
    using const_iterator = typename container::const_iterator;
    using reference = T&;
    using const_reference = const T&;
    using value_type = T;

    enumerable_thread_specific() : m_init([]() { return T(); }) {}

    template<typename F, typename std::enable_if<std::is_invocable_r<T, F>::value, int>::type = 0>
    explicit enumerable_thread_specific(F f) : m_init(std::function<T()>(f))
    {}

    template<typename U, typename std::enable_if<!std::is_invocable<U>::value && std::is_convertible<U, T>::value, int>::type = 0>
    enumerable_thread_specific(const U& exemplar) : m_init([exemplar]() { return T(exemplar); })
    {}

    enumerable_thread_specific(const enumerable_thread_specific& o) : m_init(o.m_init), m_items(o.m_items)
    {
        rebuild_index(o);
    }
    enumerable_thread_specific& operator=(const enumerable_thread_specific& o)
    {
        if (this != &o)
        {
            m_init = o.m_init;
            m_items = o.m_items;
            rebuild_index(o);
        }
        return *this;
    }
    enumerable_thread_specific(enumerable_thread_specific&& o) noexcept
        : m_init(std::move(o.m_init)), m_items(std::move(o.m_items)), m_index(std::move(o.m_index))
    {
        o.m_gen = next_gen();
    }
    enumerable_thread_specific& operator=(enumerable_thread_specific&& o) noexcept
    {
        m_init = std::move(o.m_init);
        m_items = std::move(o.m_items);
        m_index = std::move(o.m_index);
        m_gen = next_gen();
        o.m_gen = next_gen();
        return *this;
    }

    // The calling thread's element. A per-thread cache (this object, its
    // generation, the element's address - deque elements do not move) answers
    // repeated calls without the lock, as TBB's thread-local lookup does; the
    // generation changes whenever the element set is rebuilt.
    reference local()
    {
        thread_local const enumerable_thread_specific* owner = nullptr;
        thread_local std::uint64_t owner_gen = 0;
        thread_local T* cached = nullptr;
        if (owner == this && owner_gen == m_gen)
        {
            return *cached;
        }
        std::lock_guard<std::mutex> lock(m_mutex);
        const auto id = std::this_thread::get_id();
        auto found = m_index.find(id);
        T* item;
        if (found != m_index.end())
        {
            item = &m_items[found->second];
        }
        else
        {
            m_items.push_back(m_init());
            m_index[id] = m_items.size() - 1;
            item = &m_items.back();
        }
        owner = this;
        owner_gen = m_gen;
        cached = item;
        return *item;
    }

    iterator begin() { return m_items.begin(); }
    iterator end() { return m_items.end(); }
    const_iterator begin() const { return m_items.begin(); }
    const_iterator end() const { return m_items.end(); }
    std::size_t size() const { return m_items.size(); }
    bool empty() const { return m_items.empty(); }
    void clear()
    {
        m_items.clear();
        m_index.clear();
        m_gen = next_gen();
    }

private:
    void rebuild_index(const enumerable_thread_specific& o)
    {
        m_index = o.m_index;
        m_gen = next_gen();
    }
    static std::uint64_t next_gen()
    {
        static std::atomic<std::uint64_t> counter {1};
        return counter.fetch_add(1);
    }

    std::uint64_t m_gen = next_gen();

    std::function<T()> m_init;
    container m_items;
    std::map<std::thread::id, std::size_t> m_index;
    std::mutex m_mutex;
};

// Flattened view over a container of containers (the elements of every thread-local container).
template<typename Outer> class flattened2d
{
public:
    using inner_type = typename Outer::value_type;
    using value_type = typename inner_type::value_type;

    class const_iterator
    {
    public:
        using iterator_category = std::forward_iterator_tag;
        using value_type = typename inner_type::value_type;
        using difference_type = std::ptrdiff_t;
        using pointer = const value_type*;
        using reference = const value_type&;

        const_iterator(typename Outer::const_iterator o, typename Outer::const_iterator oe) : m_o(o), m_oe(oe)
        {
            if (m_o != m_oe)
            {
                m_i = m_o->begin();
                skip();
            }
        }
        reference operator*() const { return *m_i; }
        pointer operator->() const { return &*m_i; }
        const_iterator& operator++()
        {
            ++m_i;
            skip();
            return *this;
        }
        bool operator==(const const_iterator& other) const
        {
            if (m_o == m_oe || other.m_o == other.m_oe)
            {
                return (m_o == m_oe) && (other.m_o == other.m_oe);
            }
            return m_o == other.m_o && m_i == other.m_i;
        }
        bool operator!=(const const_iterator& other) const { return !(*this == other); }

    private:
        void skip()
        {
            while (m_o != m_oe && m_i == m_o->end())
            {
                ++m_o;
                if (m_o != m_oe)
                {
                    m_i = m_o->begin();
                }
            }
        }
        typename Outer::const_iterator m_o;
        typename Outer::const_iterator m_oe;
        typename inner_type::const_iterator m_i;
    };

    explicit flattened2d(const Outer& outer) : m_outer(&outer) {}
    const_iterator begin() const { return const_iterator(m_outer->begin(), m_outer->end()); }
    const_iterator end() const { return const_iterator(m_outer->end(), m_outer->end()); }

private:
    const Outer* m_outer;
};

template<typename Outer> flattened2d<Outer> flatten2d(const Outer& outer)
{
    return flattened2d<Outer>(outer);
}
}; // namespace tbb
#endif
